"""The output-file readers and the directory comparison (no GPU)."""
import numpy as np
import pytest

from chiml_gb300.outfiles import read_output, rel_l2, relative_errors


def _write_flux(path, rows):
    with open(path, "w") as f:
        f.write("#freq\tabs(incd)\treal(incd)\timag(incd)\n")
        for r in rows:
            f.write("\t".join("%.15g" % v for v in r) + "\n")


def test_reads_text_and_binary_outputs(tmp_path):
    _write_flux(tmp_path / "flux.dat", [[0.25, 1.0, 1.0, 0.0], [0.2, 2.0, 2.0, -0.5]])
    kind, hdr, v = read_output(str(tmp_path / "flux.dat"))
    assert kind == "txt" and hdr is None and v.shape == (2, 4) and v[1, 3] == -0.5
    (tmp_path / "pop.dat").write_text("0.1 0.5\n0.2 0.25\n")
    kind, _, v = read_output(str(tmp_path / "pop.dat"))
    assert kind == "txt" and np.allclose(v, [0.1, 0.5, 0.2, 0.25])
    header = np.array([2, 1, 1, 0, 0, 0], dtype=np.int32)
    payload = np.array([0.0, 1.5, -2.5], dtype=np.float64)
    (tmp_path / "box.bin").write_bytes(header.tobytes() + payload.tobytes())
    kind, hdr, v = read_output(str(tmp_path / "box.bin"))
    assert kind == "bin" and np.array_equal(hdr, header) and np.array_equal(v, payload)


def test_relative_errors_and_mismatches(tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    _write_flux(a / "f.dat", [[1.0, 2.0, 3.0, 4.0]])
    _write_flux(b / "f.dat", [[1.0, 2.0, 3.0, 4.0 + 1e-6]])
    err = relative_errors(str(a), str(b))
    assert set(err) == {"f.dat"} and 0 < err["f.dat"] < 1e-6
    assert rel_l2(np.zeros(3), np.ones(3)) == pytest.approx(np.sqrt(3.0))
    _write_flux(b / "f.dat", [[1.0, 2.0, 3.0, 4.0], [1.0, 2.0, 3.0, 4.0]])
    with pytest.raises(ValueError):
        relative_errors(str(a), str(b))
    (a / "g.dat").write_text("1 2\n")
    with pytest.raises(ValueError):
        relative_errors(str(a), str(b))
