"""Comparison of two chiML output directories with a tolerance (the readers live in chiml_gb300.outfiles)."""
from chiml_gb300.outfiles import read_output, rel_l2, relative_errors  # noqa: F401


def compare_dirs(ref_dir, out_dir, tol):
    """Compares every file under ref_dir with its counterpart; returns {relpath: rel_l2}."""
    res = relative_errors(ref_dir, out_dir)
    assert res, "no reference outputs in " + ref_dir
    for rel, e in res.items():
        assert e <= tol, "%s relative L2 %.3e > %.1e" % (rel, e, tol)
    return res
