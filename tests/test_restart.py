"""Restart files in the reference's format (host side, no GPU).

The velocity partition follows Vel_Phase_det (Hybrid2D/src/sub_init.f90:
469-560); the expected grids below were worked out by hand from that
routine.  The flag.dat sample is the reference's own
Hybrid2D/restart1/flag.dat (three list-directed values).
"""
import os
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def rs(pkg):
    from hyb_gb300 import restart
    return restart


@pytest.mark.parametrize("nprocs,khalf,nvit,nvjt,xdim,ydim", [
    (1, False, 32, 32, 1, 1),
    (2, False, 32, 32, 2, 1),
    (4, False, 32, 32, 4, 1),     # NINT(sqrt 4) - 1 = 1 divides 4
    (6, False, 32, 32, 6, 1),
    (9, False, 24, 24, 3, 3),     # 2 does not divide 9, 3 does
    (8, False, 64, 64, 4, 2),     # NINT(sqrt 8) - 1 = 2
    (4, True, 32, 32, 2, 2),      # symmetric: 2 x 2 divides both axes
    (6, True, 24, 30, 3, 2),      # YDIM 2, XDIM 3 pass every test first
])
def test_partition_grid(rs, nprocs, khalf, nvit, nvjt, xdim, ydim):
    x, y, i1, j1, ranks = rs.velocity_partition(nvit, nvjt, nprocs, khalf)
    assert (x, y) == (xdim, ydim)
    assert i1 == -(-nvit // x) and j1 == -(-nvjt // y)
    cover = np.zeros((nvit, nvjt), dtype=int)
    for ipt, iend, jpt, jend in ranks:
        assert iend <= i1 and jend <= j1
        cover[ipt:ipt + iend, jpt:jpt + jend] += 1
    assert np.all(cover == 1)


def test_partition_uneven_split(rs):
    # 32 nodes over 6 ranks: MM = 2, ranks 0-1 hold 6 nodes, ranks 2-5 hold 5
    _, _, i1, _, ranks = rs.velocity_partition(32, 16, 6)
    assert i1 == 6
    assert [(r[0], r[1]) for r in ranks] == [(0, 6), (6, 6), (12, 5), (17, 5), (22, 5), (27, 5)]


def test_partition_rejects_uneven_symmetric_split(rs):
    with pytest.raises(ValueError):
        rs.velocity_partition(30, 30, 7, khalf=True)


def test_record_markers(rs, tmp_path):
    p = tmp_path / "r.dat"
    with open(p, "wb") as fh:
        rs.write_record(fh, np.arange(5, dtype="<f8").tobytes())
    raw = p.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == 40 and struct.unpack("<i", raw[-4:])[0] == 40
    assert len(raw) == 48
    with open(p, "rb") as fh:
        assert np.array_equal(np.frombuffer(rs.read_record(fh), "<f8"), np.arange(5))


def test_subrecords(rs, tmp_path):
    p = tmp_path / "s.dat"
    data = np.random.default_rng(1).random(100).tobytes()
    with open(p, "wb") as fh:
        rs.write_record(fh, data, subrecord_max=96)
        rs.write_record(fh, b"tail")
    raw = p.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == -96            # continued
    with open(p, "rb") as fh:
        assert rs.read_record(fh) == data
        assert rs.read_record(fh) == b"tail"


def test_reference_flag_sample(rs, tmp_path):
    p = tmp_path / "flag.dat"
    p.write_text("           1\n   14.9999999999997     \n        1500\n")
    assert rs.read_flag(str(p)) == (1, 14.9999999999997, 1500)
    q = tmp_path / "flag2.dat"
    rs.write_flag(str(q), 14.9999999999997, 1500)
    assert rs.read_flag(str(q)) == (1, 14.9999999999997, 1500)


@pytest.mark.parametrize("nprocs", [1, 4, 6])
def test_round_trip(rs, tmp_path, nprocs):
    nx, ny, nvit, nvjt = 5, 9, 8, 6
    n = 2 * (nx + 7) * (ny + 7) * nvit * nvjt
    frd = np.random.default_rng(nprocs).random(n)
    rs.write(str(tmp_path), frd, nx, ny, nvit, nvjt, tt=1.25, kstep=40, slot=2, nprocs=nprocs)
    assert os.path.exists(rs.rank_file(str(tmp_path), 2, nprocs - 1))
    slot, tt, kstep, back = rs.read(str(tmp_path), nx, ny, nvit, nvjt, nprocs=nprocs)
    assert (slot, tt, kstep) == (2, 1.25, 40)
    assert np.array_equal(back, frd)


def test_slot_choice_and_missing(rs, tmp_path):
    nx, ny, nvit, nvjt = 5, 9, 4, 4
    n = 2 * (nx + 7) * (ny + 7) * nvit * nvjt
    a, b = np.ones(n), np.full(n, 2.0)
    rs.write(str(tmp_path), a, nx, ny, nvit, nvjt, 1.0, 10, slot=1)
    rs.write(str(tmp_path), b, nx, ny, nvit, nvjt, 2.0, 20, slot=2)
    assert rs.read(str(tmp_path), nx, ny, nvit, nvjt)[0] == 2      # restart2 first
    (tmp_path / "restart2" / "flag.dat").write_text("           0\n 2.0\n 20\n")
    slot, tt, kstep, f = rs.read(str(tmp_path), nx, ny, nvit, nvjt)
    assert (slot, tt, kstep) == (1, 1.0, 10) and np.all(f == 1.0)
    with pytest.raises(FileNotFoundError):
        rs.read(str(tmp_path / "none"), nx, ny, nvit, nvjt)
