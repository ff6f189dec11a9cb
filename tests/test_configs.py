"""Geometry checks of the workload generators (no GPU): the large mixed scene keeps its
structures inside the TFSF box and its flux planes clear of the film and the sheet, at the
full size and at the sizes the parity case and the FP64 crop use."""
import pytest

from chiml_gb300 import configs


def _z_extent(obj):
    half = obj["size"][2] / 2 if "size" in obj else obj.get("radius", 0.0)
    return obj["loc"][2] - half, obj["loc"][2] + half


@pytest.mark.parametrize("kw", [dict(),
                                dict(n=160, nz=80, pml=8, nell=4, film_cells=4, sheet_cells=4),
                                dict(n=40, nz=48, pml=6, nell=3, nfreq=5, sheet_cells=2, film_cells=2)])
def test_config5_layout(kw):
    cfg = configs.config5(steps=10, **kw)
    dx = cfg["CompCell"]["stepSize"][0]
    box = cfg["TFSF"][0]["size"]
    film, sheet = cfg["ObjectList"][-2], cfg["ObjectList"][-1]
    assert sheet["Basis_Set"] and not film["Basis_Set"]
    # film and sheet inside the TFSF box, with a cell of vacuum to spare
    for o in (film, sheet):
        lo, hi = _z_extent(o)
        assert -box[2] / 2 + dx < lo < hi < box[2] / 2 - dx
        assert o["size"][0] < box[0] - 2 * dx
    # three flux planes below the film, three above the sheet, all inside the box
    zs = sorted(p["loc"][2] for p in cfg["FluxList"])
    assert len(zs) == 6
    assert all(-box[2] / 2 < z < _z_extent(film)[0] for z in zs[:3])
    assert all(_z_extent(sheet)[1] < z < box[2] / 2 for z in zs[3:])
    # ellipsoid centres between the film and the sheet
    for o in cfg["ObjectList"][:-2]:
        assert _z_extent(film)[1] < o["loc"][2] < _z_extent(sheet)[0]
    # the coupling matrix is symmetric and couples adjacent levels only
    c = sheet["couplings"]
    n = len(sheet["Basis_Set"])
    for i in range(n):
        for j in range(n):
            assert c[i * n + j] == c[j * n + i]
            assert (c[i * n + j] != 0) == (abs(i - j) == 1)
