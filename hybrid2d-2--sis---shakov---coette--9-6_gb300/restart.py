"""Restart files of the reference solver, read and written from the host.

The reference backs up the distribution function with backup_Macro_write /
backup_Mesco_write and restarts with init_flow_read / backup_Mesco_read
(Hybrid2D/src/Backup_write_read.f90:1-56, :56-112, :114-148, :150-209):

    restart<slot>/flag.dat                 list-directed text: 1, tt, Kstep
    restart<slot>/star<NN>/restart<MMMMM>.dat
                                           one file per MPI rank (NN = rank
                                           / 1024, MMMMM = rank), one
                                           unformatted sequential record per
                                           kinetic block holding
                                           B%FRD(NRD,-3:nx+3,-3:ny+3,I1MAX,J1MAX)
                                           in REAL(8), column-major

Each rank holds a block of the velocity grid (Vel_Phase_det,
Hybrid2D/src/sub_init.f90:469-560): the ranks form an XDIM x YDIM grid over
(NVIT, NVJT); rank r = x + XDIM y holds the nodes iv + IPT, jv + JPT for
iv = 1..IEND, jv = 1..JEND, in FRD slots of a common I1MAX x J1MAX size (the
slots past IEND / JEND are allocated but unused; they are written as zeros).
init_flow_read takes restart2 when its flag is 1, else restart1.

Records use the 4-byte length markers of unformatted sequential files.  A
record longer than 2**31 - 9 bytes is split into subrecords whose head and
tail markers are negative for every subrecord but the last (the gfortran
convention; Intel Fortran writes the same layout for such records with its
sign-bit continuation flag).

The single-GPU solver holds all velocities, so `read` assembles the global
FRD(NRD,-3:nx+3,-3:ny+3,NVIT,NVJT) that hyb_upload_f takes, and `write`
splits the array hyb_download_f returns over the ranks of the run that is
to read it.
"""
import math
import os
import struct

import numpy as np

NRD = 2
LAP = 3
SUBRECORD_MAX = 2 ** 31 - 9


def velocity_partition(nvit, nvjt, nprocs, khalf=False):
    """Vel_Phase_det: (XDIM, YDIM, I1MAX, J1MAX, [(IPT, IEND, JPT, JEND)
    per rank]).  khalf is set when a block has a symmetry or sliding-wall
    face (Hybrid2D/src/sub_init.f90:246-281)."""
    if nprocs < 1:
        raise ValueError("nprocs must be >= 1")
    if khalf:
        if (nvit * nvjt) % nprocs != 0:
            raise ValueError("khalf: NVIT*NVJT must be a multiple of the rank count")
        ydim = int(round(math.sqrt(nprocs))) - 1
        xdim = 0
        for _ in range(1, nprocs - ydim + 1):
            ydim += 1
            xdim = nprocs // ydim
            if (nprocs % ydim == 0 and nprocs % xdim == 0 and nvit % xdim == 0 and nvjt % ydim == 0
                    and xdim * ydim == nprocs):
                break
        if nvit % xdim != 0 or nvjt % ydim != 0:
            xdim = int(round(math.sqrt(nprocs))) - 1
            for _ in range(1, nprocs - xdim + 1):
                xdim += 1
                ydim = nprocs // xdim
                if (nprocs % ydim == 0 and nprocs % xdim == 0 and nvit % xdim == 0 and nvjt % ydim == 0
                        and xdim * ydim == nprocs):
                    break
        if nprocs != 1 and (nvit % xdim != 0 or nvjt % ydim != 0):
            raise ValueError("khalf: the velocity grid does not split evenly over the ranks")
    else:
        ydim = int(round(math.sqrt(nprocs))) - 1
        for _ in range(1, nprocs - ydim + 1):
            if ydim > 0 and nprocs % ydim == 0:
                break
            ydim += 1
        xdim = nprocs // ydim
    if xdim * ydim != nprocs:
        raise ValueError("the rank count does not factor into a velocity-space grid")
    i1max = (nvit + xdim - 1) // xdim
    j1max = (nvjt + ydim - 1) // ydim
    ranks = []
    for r in range(nprocs):
        x, y = r % xdim, r // xdim
        mm = nvit % xdim
        if x < mm:
            iend = nvit // xdim + 1
            ipt = x * iend
        else:
            iend = nvit // xdim
            ipt = x * iend + mm
        mm = nvjt % ydim
        if y < mm:
            jend = nvjt // ydim + 1
            jpt = y * jend
        else:
            jend = nvjt // ydim
            jpt = y * jend + mm
        ranks.append((ipt, iend, jpt, jend))
    return xdim, ydim, i1max, j1max, ranks


def rank_file(root, slot, rank):
    return os.path.join(root, "restart%d" % slot, "star%02d" % (rank // 1024), "restart%05d.dat" % rank)


# ---- unformatted sequential records ---------------------------------------
def write_record(fh, payload, subrecord_max=SUBRECORD_MAX):
    mv = memoryview(payload).cast("B")
    n = len(mv)
    pos = 0
    while True:
        k = min(subrecord_max, n - pos)
        last = pos + k == n
        m = k if last else -k
        fh.write(struct.pack("<i", m))
        fh.write(mv[pos:pos + k])
        fh.write(struct.pack("<i", m))
        pos += k
        if last:
            return


def read_record(fh):
    parts = []
    while True:
        head = fh.read(4)
        if len(head) < 4:
            raise EOFError("no record at this position")
        (m,) = struct.unpack("<i", head)
        k = -m if m < 0 else m
        data = fh.read(k)
        (t,) = struct.unpack("<i", fh.read(4))
        if len(data) != k or t != m:
            raise ValueError("corrupt record markers (%d / %d, %d bytes)" % (m, t, len(data)))
        parts.append(data)
        if m >= 0:
            return b"".join(parts)


# ---- flag.dat ---------------------------------------------------------------
def write_flag(path, tt, kstep, flag=1):
    """List-directed output of `write(110,*) 1 / tt / Kstep`."""
    with open(path, "w") as fh:
        fh.write("%12d\n" % flag)
        fh.write("   %-21.15g\n" % tt)
        fh.write("%12d\n" % kstep)


def read_flag(path):
    """(flag, tt, Kstep) as init_flow_read reads them (one value per line)."""
    with open(path) as fh:
        vals = [ln.split() for ln in fh if ln.strip()]
    flag = int(vals[0][0])
    tt = float(vals[1][0].replace("D", "E").replace("d", "e"))
    kstep = int(vals[2][0])
    return flag, tt, kstep


# ---- FRD ---------------------------------------------------------------------
def _frd_shape(nx, ny, n1, n2):
    return (NRD, nx + 2 * LAP + 1, ny + 2 * LAP + 1, n1, n2)


def write(root, frd, nx, ny, nvit, nvjt, tt, kstep, slot=1, nprocs=1, khalf=False,
          subrecord_max=SUBRECORD_MAX):
    """Back up the global FRD (the flat column-major array of hyb_download_f)
    for a run on `nprocs` ranks, as backup_Macro_write(slot) does."""
    full = np.asarray(frd, dtype=np.float64).reshape(_frd_shape(nx, ny, nvit, nvjt), order="F")
    _, _, i1max, j1max, ranks = velocity_partition(nvit, nvjt, nprocs, khalf)
    for r, (ipt, iend, jpt, jend) in enumerate(ranks):
        blk = np.zeros(_frd_shape(nx, ny, i1max, j1max), dtype="<f8", order="F")
        blk[:, :, :, :iend, :jend] = full[:, :, :, ipt:ipt + iend, jpt:jpt + jend]
        path = rank_file(root, slot, r)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as fh:
            write_record(fh, blk.tobytes(order="F"), subrecord_max)
    write_flag(os.path.join(root, "restart%d" % slot, "flag.dat"), tt, kstep)


def read(root, nx, ny, nvit, nvjt, nprocs=1, khalf=False, slot=None):
    """Restart as init_flow_read does: (slot, tt, Kstep, flat global FRD)."""
    if slot is None:
        slot = None
        for s in (2, 1):
            p = os.path.join(root, "restart%d" % s, "flag.dat")
            if os.path.exists(p) and read_flag(p)[0] == 1:
                slot = s
                break
        if slot is None:
            raise FileNotFoundError("no backup data is available")
    _, tt, kstep = read_flag(os.path.join(root, "restart%d" % slot, "flag.dat"))
    _, _, i1max, j1max, ranks = velocity_partition(nvit, nvjt, nprocs, khalf)
    full = np.zeros(_frd_shape(nx, ny, nvit, nvjt), dtype=np.float64, order="F")
    shape = _frd_shape(nx, ny, i1max, j1max)
    nbytes = 8 * int(np.prod(shape))
    for r, (ipt, iend, jpt, jend) in enumerate(ranks):
        with open(rank_file(root, slot, r), "rb") as fh:
            rec = read_record(fh)
        if len(rec) != nbytes:
            raise ValueError("rank %d: record of %d bytes, expected %d" % (r, len(rec), nbytes))
        blk = np.frombuffer(rec, dtype="<f8").reshape(shape, order="F")
        full[:, :, :, ipt:ipt + iend, jpt:jpt + jend] = blk[:, :, :, :iend, :jend]
    return slot, tt, kstep, full.reshape(-1, order="F")
