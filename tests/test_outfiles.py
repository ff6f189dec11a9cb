"""The output-file readers and the per-column directory comparison (no GPU)."""
import numpy as np
import pytest

from chiml_gb300.outfiles import column_errors, error_summary, read_output, rel_l2, relative_errors


def _write_flux(path, rows):
    with open(path, "w") as f:
        f.write("#" + "%16s" % "freq\tabs(incd)\treal(incd)\timag(incd)" + "freq\tabs(total)\treal(total)\timag(total)\n")
        for r in rows:
            f.write("\t".join("%.15g" % v for v in r) + "\n")


def _write_txt_detector(path, rows):
    with open(path, "w") as f:
        f.write("# time\tx\ty\tz\tfield\n")
        for r in rows:
            f.write("\t".join("%.18g" % v for v in r) + "\n")


def test_reads_text_and_binary_outputs(tmp_path):
    _write_flux(tmp_path / "flux.dat", [[0.25, 1.0, 1.0, 0.0, 2.0, 2.0, 0.0], [0.2, 2.0, 2.0, -0.5, 1.0, 1.0, 0.0]])
    kind, hdr, v = read_output(str(tmp_path / "flux.dat"))
    assert kind == "txt" and hdr.startswith("#") and v.shape == (2, 7) and v[1, 3] == -0.5
    (tmp_path / "pop.dat").write_text("0.1 0.5 0 0.5\n0.2 0.25 0 0.25\n")
    kind, hdr, v = read_output(str(tmp_path / "pop.dat"))
    assert kind == "txt" and hdr is None and np.allclose(v, [[0.1, 0.5, 0, 0.5], [0.2, 0.25, 0, 0.25]])
    header = np.array([2, 1, 1, 0, 0, 0], dtype=np.int32)
    payload = np.array([0.0, 1.5, -2.5], dtype=np.float64)
    (tmp_path / "box.bin").write_bytes(header.tobytes() + payload.tobytes())
    kind, hdr, v = read_output(str(tmp_path / "box.bin"))
    assert kind == "bin" and np.array_equal(hdr, header) and np.array_equal(v, payload)


def test_flux_error_of_one_face_is_not_diluted_by_the_frequency_column(tmp_path):
    """A flux spectrum of O(1e-10) next to a frequency column of O(1): a 1e-3 error in the
    total flux must show as 1e-3, not as the ~1e-13 a whole-file norm would report."""
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    f = np.linspace(0.25, 0.2, 20)
    flux = 1e-10 * (1.0 + np.sin(30 * f))
    rows_a = [[fr, 0, 0, 0, v, v, 0] for fr, v in zip(f, flux)]
    rows_b = [[fr, 0, 0, 0, v * (1 + 1e-3), v * (1 + 1e-3), 0] for fr, v in zip(f, flux)]
    _write_flux(a / "flux.dat", rows_a)
    _write_flux(b / "flux.dat", rows_b)
    whole = rel_l2(np.array(rows_a), np.array(rows_b))
    assert whole < 1e-11
    err = relative_errors(str(a), str(b))
    assert err["flux.dat"] == pytest.approx(1e-3, rel=1e-6)
    det = relative_errors(str(a), str(b), detail=True)["flux.dat"]
    assert det["triple0"] == 0.0 and det["triple1"] == pytest.approx(1e-3, rel=1e-6)
    assert error_summary(str(a), str(b))["flux"] == pytest.approx(1e-3, rel=1e-6)


def test_detector_error_is_not_diluted_by_the_time_column(tmp_path):
    t = np.arange(100) * 0.025
    ez = 3e-4 * np.sin(t)
    _write_txt_detector(tmp_path / "a.dat", [[ti, 0.85, 0, 0.05, v] for ti, v in zip(t, ez)])
    _write_txt_detector(tmp_path / "b.dat", [[ti, 0.85, 0, 0.05, v * 1.01] for ti, v in zip(t, ez)])
    e = column_errors(str(tmp_path / "a.dat"), str(tmp_path / "b.dat"))
    assert e["points"] == pytest.approx(1e-2, rel=1e-6)


def test_binary_detector_compares_the_payload_without_time(tmp_path):
    header = np.array([2, 1, 1, 0, 0, 0], dtype=np.int32)
    a = np.array([0.0, 1.0, 2.0, 1.0, 3.0, 4.0])  # two samples: t, two points
    b = a.copy()
    b[[1, 2, 4, 5]] *= 1.001
    (tmp_path / "a.bin").write_bytes(header.tobytes() + a.tobytes())
    (tmp_path / "b.bin").write_bytes(header.tobytes() + b.tobytes())
    e = column_errors(str(tmp_path / "a.bin"), str(tmp_path / "b.bin"))
    assert list(e) == ["points"] and e["points"] == pytest.approx(1e-3, rel=1e-6)
    c = a.copy()
    c[3] = 1.5  # a different time stamp
    (tmp_path / "c.bin").write_bytes(header.tobytes() + c.tobytes())
    with pytest.raises(ValueError, match="coordinate"):
        column_errors(str(tmp_path / "a.bin"), str(tmp_path / "c.bin"))


def test_emitter_files_take_time_as_the_coordinate(tmp_path):
    (tmp_path / "a_level_0.dat").write_text("0\t1\t0\t1\n0.5\t0.9\t0\t0.9\n")
    (tmp_path / "b_level_0.dat").write_text("0\t1\t0\t1\n0.5\t0.9009\t0\t0.9009\n")
    e = column_errors(str(tmp_path / "a_level_0.dat"), str(tmp_path / "b_level_0.dat"))
    assert e["values"] == pytest.approx(rel_l2([[1, 0, 1], [0.9, 0, 0.9]], [[1, 0, 1], [0.9009, 0, 0.9009]]))


def test_relative_errors_and_mismatches(tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    _write_flux(a / "f.dat", [[1.0, 2.0, 3.0, 4.0, 1, 1, 0]])
    _write_flux(b / "f.dat", [[1.0, 2.0, 3.0, 4.0 + 1e-6, 1, 1, 0]])
    err = relative_errors(str(a), str(b))
    assert set(err) == {"f.dat"} and 0 < err["f.dat"] < 1e-6
    assert rel_l2(np.zeros(3), np.ones(3)) == pytest.approx(np.sqrt(3.0))
    _write_flux(b / "f.dat", [[1.0, 2.0, 3.0, 4.0, 1, 1, 0], [1.0, 2.0, 3.0, 4.0, 1, 1, 0]])
    with pytest.raises(ValueError):
        relative_errors(str(a), str(b))
    _write_flux(b / "f.dat", [[1.5, 2.0, 3.0, 4.0, 1, 1, 0]])
    with pytest.raises(ValueError, match="coordinate"):
        relative_errors(str(a), str(b))
    _write_flux(b / "f.dat", [[1.0, 2.0, 3.0, 4.0, 1, 1, 0]])
    (a / "g.dat").write_text("1 2\n")
    with pytest.raises(ValueError):
        relative_errors(str(a), str(b))


def test_flux_fields_files_compare_per_face(tmp_path):
    """Saved flux fields: the integer header must agree exactly; the four grids of a face
    (Ej, Ek, Hj, Hk, stored field by field over all faces) are one group, so an error in a
    grid that is small next to its face's other grids is weighed against the face."""
    def write(path, grids, nf=2, faces=2):
        ints = [nf, 3, 3, 3] + [faces] * 4
        body = b""
        for g in grids:
            body += np.array([nf, 1, len(g) // nf], dtype=np.int32).tobytes() + np.asarray(g, dtype=np.complex128).tobytes()
        path.write_bytes(np.array(ints, dtype=np.int32).tobytes() + body)
    rng = np.random.default_rng(3)
    g = [rng.normal(size=4) + 1j * rng.normal(size=4) for _ in range(8)]
    g[5] = g[5] * 1e-3                      # face 1's Hj: near zero
    write(tmp_path / "a_fields.dat", g)
    h = [x.copy() for x in g]
    h[5] = h[5] * (1 + 1e-2)
    write(tmp_path / "b_fields.dat", h)
    e = column_errors(str(tmp_path / "a_fields.dat"), str(tmp_path / "b_fields.dat"))
    assert list(e) == ["face0", "face1"] and e["face0"] == 0.0
    face1 = np.concatenate([g[1], g[3], g[5], g[7]])
    assert e["face1"] == pytest.approx(np.linalg.norm(g[5]) * 1e-2 / np.linalg.norm(face1), rel=1e-6)
    h[3] = h[3] * (1 + 1e-3)                # a 1e-3 error in face 1's Ek shows as ~1e-3
    write(tmp_path / "c_fields.dat", h)
    e = column_errors(str(tmp_path / "a_fields.dat"), str(tmp_path / "c_fields.dat"))
    assert 1e-4 < e["face1"] < 1e-3
    write(tmp_path / "d_fields.dat", g, nf=1)
    with pytest.raises(ValueError):
        column_errors(str(tmp_path / "a_fields.dat"), str(tmp_path / "d_fields.dat"))
