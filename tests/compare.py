"""Comparison of two chiML output directories with a tolerance, per data column group (the
readers and the column layouts live in chiml_gb300.outfiles)."""
from chiml_gb300.outfiles import read_output, rel_l2, relative_errors  # noqa: F401


def compare_dirs(ref_dir, out_dir, tol):
    """Compares every file under ref_dir with its counterpart, each data group (spectrum
    triple, detector points, emitter values) on its own; returns {relpath: worst rel_l2}."""
    det = relative_errors(ref_dir, out_dir, detail=True)
    assert det, "no reference outputs in " + ref_dir
    res = {}
    for rel, groups in det.items():
        for g, e in groups.items():
            assert e <= tol, "%s [%s] relative L2 %.3e > %.1e" % (rel, g, e, tol)
        res[rel] = max(groups.values(), default=0.0)
    return res
