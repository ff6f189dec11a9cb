"""Readers and comparisons for chiML output files (text detectors, binary detectors, flux spectra)."""
import os

import numpy as np


def read_output(path):
    """Returns (kind, header, values) for a detector or flux file."""
    raw = open(path, "rb").read()
    if raw[:1] == b"#":
        rows = [l.split() for l in raw.decode().splitlines() if not l.startswith("#")]
        return "txt", None, np.array([[float(x) for x in r] for r in rows])
    try:
        # headerless numeric text: emitter population and polarisation files
        rows = [l.split() for l in raw.decode("ascii").splitlines() if l.strip()]
        return "txt", None, np.array([float(x) for r in rows for x in r])
    except (UnicodeDecodeError, ValueError):
        pass
    hdr = np.frombuffer(raw[:24], dtype=np.int32)
    return "bin", hdr, np.frombuffer(raw[24:], dtype=np.float64)


def rel_l2(a, b):
    den = np.linalg.norm(a)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def compare_dirs(ref_dir, out_dir, tol):
    """Compares every file under ref_dir with its counterpart; returns {relpath: rel_l2}."""
    res = {}
    for d, _, files in os.walk(ref_dir):
        for f in files:
            p = os.path.join(d, f)
            rel = os.path.relpath(p, ref_dir)
            q = os.path.join(out_dir, rel)
            assert os.path.exists(q), "missing output " + rel
            ka, ha, a = read_output(p)
            kb, hb, b = read_output(q)
            assert ka == kb, rel
            if ha is not None:
                assert np.array_equal(ha, hb), rel
            assert a.shape == b.shape, "%s: %s vs %s" % (rel, a.shape, b.shape)
            e = rel_l2(a, b)
            res[rel] = e
            assert e <= tol, "%s relative L2 %.3e > %.1e" % (rel, e, tol)
    assert res, "no reference outputs in " + ref_dir
    return res
