"""The reader of the reference's text field dumps (carpio_gb300.dump, the
interface of pyscript/read.py) on the reference's own Output_Scalar files
(ops_* fixtures: dump.txt written by s_io_file.hpp:43-71 from in_a)."""
import numpy as np
import pytest

from conftest import golden, golden_names


@pytest.mark.parametrize("name", golden_names("ops_"))
def test_reader_on_reference_dump(name, tmp_path):
    from carpio_gb300 import dump
    d = golden(name)
    if "dump_text" not in d:
        pytest.skip("fixture without a dump")
    nx, ny, gl = int(d["nx"]), int(d["ny"]), int(d["gl"])
    f = tmp_path / "ref.txt"
    f.write_bytes(d["dump_text"].tobytes())
    t = dump.TextFile(str(f))
    c = t.get_config()
    assert (int(c["NX"]), int(c["NY"]), int(c["Dim"]), int(c["Size"])) == (nx, ny, 2, nx * ny)
    a = d["in_a"][gl:gl + nx, gl:gl + ny]
    # %10.6e: 7 significant digits
    assert np.allclose(t.field(), a, rtol=1e-6, atol=1e-6)
    assert np.allclose(t.get_coo_x(), d["grid_cx"][gl:gl + nx], rtol=1e-6)
    assert np.allclose(t.get_coo_y(), d["grid_cy"][gl:gl + ny], rtol=1e-6)
    assert len(t.get_mat_val()) == ny and len(t.get_mat_val()[0]) == nx
    assert dump.diff(str(f), str(f)) == 0.0
    # a changed value shows in the difference
    lines = f.read_text().splitlines(keepends=True)
    k = next(i for i, ln in enumerate(lines) if not ln.startswith("#"))
    parts = lines[k].split(",")
    parts[3] = " %10.6e\n" % (float(parts[3]) + 0.5)
    lines[k] = ",".join(parts)
    g2 = tmp_path / "changed.txt"
    g2.write_text("".join(lines))
    assert abs(dump.diff(str(f), str(g2)) - 0.5) < 1e-5
