"""Readers for chiML's output files (text detectors, flux spectra, emitter population and
polarisation files, binary detectors) and a per-file relative-error comparison of two
output directories."""
import os

import numpy as np


def read_output(path):
    """Returns (kind, header, values) for a detector or flux file: kind "txt" with the numbers
    of a text file (rows of a '#'-headed file, or every number of a headerless one), or "bin"
    with the 6-int header and the FP64 payload of a binary detector."""
    raw = open(path, "rb").read()
    if raw[:1] == b"#":
        rows = [l.split() for l in raw.decode().splitlines() if not l.startswith("#")]
        return "txt", None, np.array([[float(x) for x in r] for r in rows])
    try:
        rows = [l.split() for l in raw.decode("ascii").splitlines() if l.strip()]
        return "txt", None, np.array([float(x) for r in rows for x in r])
    except (UnicodeDecodeError, ValueError):
        pass
    hdr = np.frombuffer(raw[:24], dtype=np.int32)
    return "bin", hdr, np.frombuffer(raw[24:], dtype=np.float64)


def rel_l2(a, b):
    """||a - b|| / ||a|| (the absolute norm when a is zero)."""
    den = np.linalg.norm(a)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def relative_errors(ref_dir, out_dir):
    """{relative path: rel_l2(ref, out)} for every file under ref_dir. Raises ValueError when
    a file is missing on the out_dir side or its kind, header or shape differ."""
    res = {}
    for d, _, files in os.walk(ref_dir):
        for f in files:
            p = os.path.join(d, f)
            rel = os.path.relpath(p, ref_dir)
            q = os.path.join(out_dir, rel)
            if not os.path.exists(q):
                raise ValueError("missing output " + rel)
            ka, ha, a = read_output(p)
            kb, hb, b = read_output(q)
            if ka != kb or (ha is not None and not np.array_equal(ha, hb)) or a.shape != b.shape:
                raise ValueError("%s: kind, header or shape differ (%s vs %s)" % (rel, a.shape, b.shape))
            res[rel] = rel_l2(a, b)
    return res
