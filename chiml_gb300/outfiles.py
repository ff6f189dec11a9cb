"""Readers for chiML's output files and a per-column relative-error comparison of two output
directories.

The files and their column layouts (what is a coordinate and what is data):

* text detectors (`DTC/parallelDTC_TXT.cpp:20-53`): header ``# time x y z field``, then one
  row per sample: t, x, y, z, and the values of every point of the box;
* binary detectors (`DTC/parallelDTC_BIN.cpp:12-50`): six int32 (box size, location), then
  per sample t and sz[0]*sz[1]*sz[2] FP64 values;
* flux spectra (`DTC/parallelFlux.hpp:444-540`): header ``#freq ...``, then per frequency the
  frequency and (abs, real, imag) triples: incident, each face, total;
* frequency-domain detectors (`DTC/parallelDTC_FREQ.hpp:390-450`): ``#freq ...`` files with
  triples (incident fields, their sum, each field, the total), and per-frequency maps
  ``#x y z ...`` with three coordinate columns before the triples;
* emitter populations (`ML/QEPopDtc.cpp:37-61`): headerless rows t, re, im, abs;
* emitter polarisation (`ML/parallelQE.cpp:520-557`): headerless rows t, then Px, Py and/or
  Pz and |P|;
* saved flux fields (`DTC/parallelFlux.hpp:616-660`, `<flux>_fields.dat`): integers (sizes)
  that must agree exactly, and one complex grid per face and field (all faces' Ej, then Ek,
  Hj, Hk); the four grids of a face, from which its flux is formed, are one data group.

The comparison leaves coordinates out of the error (they must agree, or the files do not
describe the same samples) and takes the relative L2 error of every data group on its own:
each (abs, real, imag) triple of the spectra, the point values of a detector, the population
triple, the polarisation columns. A file's error is the worst group's, so a small column
is not hidden by a large one (a time column of O(100) next to fields of O(1e-4), a
frequency column next to fluxes of O(1e-10)).
"""
import os

import numpy as np

COORD_TOL = 1e-9  # coordinate columns (time, x/y/z, frequency) must agree to this relative L2


def read_flux_fields(raw):
    """(ints, [complex grids]) of a flux fields file (parallelFluxDTC::saveFields,
    DTC/parallelFlux.hpp:616-660): int nfreq and the flux size (4 ints), the number of faces of
    each of Ej, Ek, Hj, Hk (4 ints), then per grid its 3-int size and its complex values."""
    head = np.frombuffer(raw[:32], dtype=np.int32)
    ints = list(head)
    grids = []
    pos = 32
    for _ in range(int(head[4:8].sum())):
        n = np.frombuffer(raw[pos:pos + 12], dtype=np.int32)
        ints.extend(int(v) for v in n)
        pos += 12
        cnt = int(np.prod(n))
        grids.append(np.frombuffer(raw[pos:pos + 16 * cnt], dtype=np.complex128))
        pos += 16 * cnt
    if pos != len(raw):
        raise ValueError("flux fields file of unexpected length")
    return np.array(ints, dtype=np.int64), grids


def read_output(path):
    """Returns (kind, header, values): kind "txt" with the header line (None for headerless
    files) and the rows of a text file as a 2-D array; kind "bin" with the six-int header
    and the FP64 payload of a binary detector; or kind "fields" with the integers and the
    complex grids of a saved flux fields file."""
    raw = open(path, "rb").read()
    if path.endswith("_fields.dat"):
        ints, grids = read_flux_fields(raw)
        return "fields", ints, grids
    try:
        text = raw.decode("ascii")
    except UnicodeDecodeError:
        text = None
    if text is not None:
        header = None
        rows = []
        ok = True
        for line in text.splitlines():
            if line.startswith("#"):
                if header is None:
                    header = line
                continue
            if not line.strip():
                continue
            try:
                rows.append([float(x) for x in line.split()])
            except ValueError:
                ok = False
                break
        if ok and (header is not None or rows):
            width = max((len(r) for r in rows), default=0)
            if any(len(r) != width for r in rows):
                raise ValueError("%s: ragged rows" % path)
            return "txt", header, np.array(rows, dtype=np.float64).reshape(len(rows), width)
    hdr = np.frombuffer(raw[:24], dtype=np.int32)
    return "bin", hdr, np.frombuffer(raw[24:], dtype=np.float64)


def rel_l2(a, b):
    """||a - b|| / ||a|| (the absolute norm when a is zero)."""
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = np.asarray(a, dtype=dt)
    b = np.asarray(b, dtype=dt)
    den = np.linalg.norm(a)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def fields_groups(ints, grids):
    """[(group name, values)] of a flux fields file: per face the concatenation of its Ej, Ek,
    Hj and Hk grids. A face's flux is Re(Ej Hk* - Ek Hj*) summed over the face, so a grid
    that is near zero by symmetry (3e-3 next to 1.5 on the same face) counts against its
    face's field, not against its own size. Files whose four field counts differ are
    compared per grid."""
    counts = [int(v) for v in ints[4:8]]
    n = counts[0]
    if n == 0 or counts != [n] * 4 or len(grids) != 4 * n:
        return [("grid%d" % k, g) for k, g in enumerate(grids)]
    return [("face%d" % f, np.concatenate([grids[f + k * n] for k in range(4)])) for f in range(n)]


def split_columns(kind, header, values):
    """(coordinates, [(group name, data array)]) of one parsed output file."""
    if kind == "fields":
        return header.astype(np.float64), fields_groups(header, values)
    if kind == "bin":
        npts = int(np.prod(header[:3])) if header.size >= 3 else 0
        rec = npts + 1
        if npts <= 0 or values.size % rec:
            return None, [("payload", values)]
        v = values.reshape(-1, rec)
        return v[:, 0], [("points", v[:, 1:])]
    v = values
    if v.ndim != 2 or v.shape[1] == 0:
        return None, [("values", v)]
    h = (header or "").lstrip("#").strip()
    if h.startswith("time"):                    # text detector: t, x, y, z, point values
        return v[:, :4], [("points", v[:, 4:])]
    if h.startswith("x"):                       # frequency map: x, y, z, triples
        ncoord = 3
    elif h.startswith("freq"):                  # flux spectrum / frequency detector: f, triples
        ncoord = 1
    else:                                       # headerless emitter files: t, then values
        return v[:, :1], [("values", v[:, 1:])]
    data = v[:, ncoord:]
    if data.shape[1] % 3:
        return v[:, :ncoord], [("values", data)]
    return v[:, :ncoord], [("triple%d" % (k // 3), data[:, k:k + 3]) for k in range(0, data.shape[1], 3)]


def column_errors(ref_path, out_path):
    """{group name: relative L2} of one file against its reference. Raises ValueError when the
    kinds, headers, shapes or coordinate columns differ."""
    ka, ha, a = read_output(ref_path)
    kb, hb, b = read_output(out_path)
    if ka == "fields" and kb == "fields":
        if not np.array_equal(ha, hb) or len(a) != len(b):
            raise ValueError("%s: flux fields header or grid sizes differ" % out_path)
        return {name: rel_l2(x, y) for (name, x), (_, y) in zip(fields_groups(ha, a), fields_groups(hb, b))}
    if ka != kb or getattr(a, "shape", None) != getattr(b, "shape", None):
        raise ValueError("%s: kind or shape differ (%s vs %s)" % (out_path, a.shape, b.shape))
    if ka == "bin" and not np.array_equal(ha, hb):
        raise ValueError("%s: binary header differs" % out_path)
    ca, ga = split_columns(ka, ha, a)
    cb, gb = split_columns(kb, hb, b)
    if ca is not None and rel_l2(ca, cb) > COORD_TOL:
        raise ValueError("%s: coordinate columns differ (relative L2 %.3e)" % (out_path, rel_l2(ca, cb)))
    return {name: rel_l2(x, y) for (name, x), (_, y) in zip(ga, gb)}


def relative_errors(ref_dir, out_dir, detail=False):
    """{relative path: worst data-group relative L2} for every file under ref_dir (with
    detail=True, {relative path: {group: relative L2}}). Raises ValueError when a file is
    missing on the out_dir side or its kind, header, shape or coordinates differ."""
    res = {}
    for d, _, files in os.walk(ref_dir):
        for f in files:
            p = os.path.join(d, f)
            rel = os.path.relpath(p, ref_dir)
            q = os.path.join(out_dir, rel)
            if not os.path.exists(q):
                raise ValueError("missing output " + rel)
            errs = column_errors(p, q)
            res[rel] = errs if detail else max(errs.values(), default=0.0)
    return res


def file_class(rel):
    """'flux', 'emitter' or 'field' for an output file name (for error summaries)."""
    name = os.path.basename(rel)
    if "flux" in name:
        return "flux"
    if "_level_" in name or "pol" in name:
        return "emitter"
    return "field"


def error_summary(ref_dir, out_dir):
    """Worst relative L2 per class of output file: {"fields", "flux", "populations"} (None
    where a class has no file)."""
    worst = {"field": None, "flux": None, "emitter": None}
    for rel, e in relative_errors(ref_dir, out_dir).items():
        c = file_class(rel)
        worst[c] = e if worst[c] is None else max(worst[c], e)
    return {"fields": worst["field"], "flux": worst["flux"], "populations": worst["emitter"]}
