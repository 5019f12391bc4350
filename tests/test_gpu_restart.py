"""A GPU run backed up in the reference's restart format and resumed.

hyb_download_f -> restart files of a 4-rank run -> restart read ->
hyb_upload_f into a new context: the resumed run continues exactly as the
original (FP64, bit-identical f after further steps).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_backup_and_resume(pkg, tmp_path):
    from hyb_gb300 import abi, cases, restart
    c = cases.couette_small(ncy=32, nvx=16, nvy=16, dt=0.05)
    a = abi.Solver(c, precision=0)
    a.init_maxwellian()
    a.step(5)
    restart.write(str(tmp_path), a.download_f(), c.nx, c.ny, c.nvx, c.nvy, tt=0.25, kstep=5, slot=1, nprocs=4)
    slot, tt, kstep, frd = restart.read(str(tmp_path), c.nx, c.ny, c.nvx, c.nvy, nprocs=4)
    assert (slot, tt, kstep) == (1, 0.25, 5)
    b = abi.Solver(c, precision=0)
    b.upload_f(frd)
    assert np.array_equal(b.download_f(), a.download_f())
    a.step(3)
    b.step(3)
    assert np.array_equal(b.download_f(), a.download_f())
    assert np.array_equal(b.moments()[0], a.moments()[0])
