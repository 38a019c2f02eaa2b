"""Parameter files (writeToFile / readFromFile, src/goofit/FunctorWriter.cpp:9-62): a written file
restores every parameter's value, error and limits exactly; lines naming other parameters are skipped."""
import goofit_gb300 as gf
from goofit_gb300 import workloads as W


def test_write_then_read_restores_the_parameters(tmp_path):
    wl = W.make_c2(1000)
    params = wl.pdf.getParameters()
    saved = {v.getName(): (v.value, v.error, v.lowerlimit, v.upperlimit) for v in params}
    f = tmp_path / "params.txt"
    gf.writeToFile(wl.pdf, str(f))
    lines = f.read_text().splitlines()
    assert len(lines) == len(params) and all(len(l.split()) == 5 for l in lines)
    for v in params:
        v.setValue(v.value * 0.5 + 0.1)
        v.setError(1.0)
    f.write_text("unknown_parameter 1 2 3 4\n" + f.read_text())
    gf.readFromFile(wl.pdf, str(f))
    for v in params:
        assert (v.value, v.error, v.lowerlimit, v.upperlimit) == saved[v.getName()]


def test_read_list_of_numbers(tmp_path):
    f = tmp_path / "n.txt"
    f.write_text("1 2.5\n-3e-2\n")
    assert gf.readListOfNumbers(str(f)) == [1.0, 2.5, -0.03]
