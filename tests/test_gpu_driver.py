"""The command-line driver end to end on Rutherford-Boeing files."""
import numpy as np
import pytest

from spral_gb300 import driver, matrices as M, rb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("args,shift", [(["--nrhs=2"], -0.4), (["--pos"], 0.5),
                                        (["--mixed"], -0.4), (["--scale=equil"], -0.4)])
def test_gpu_driver_reports_solution(tmp_path, capsys, args, shift):
    p, r, v = M.laplacian_3d(10, shift=shift)
    f = tmp_path / "m.rb"
    rb.rb_write(str(f), p, r, v, "rsa", title="3D Laplacian 10^3")
    assert driver.main(args + [str(f)]) == 0
    out = capsys.readouterr().out
    bwd = [float(x) for x in out.split("bwd error scaled =")[1].split("\n")[0].split()]
    assert max(bwd) <= 1e-13
    neg = int(out.split("inertia:")[1].split()[0])
    expect = 0 if "--pos" in args else M.laplacian_eig_count_3d(10, 10, 10, shift)[0]
    assert neg == expect
