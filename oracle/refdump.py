"""Reader for the raw FP64 dumps written by the reference-side dump module
(oracle/ref/nmgdump/nmgdump.c).  Test infrastructure only.

Each element record holds: patch index, n[3], (v2: the finite-volume
flag use_fv), bbox[6] and the arrays x, y, z, dXdx[9], sqrtgdiag[3],
(v2: det_dXbdx), u[5] (pi, cx, cy, cz, phi) and optionally r[5] = RHS(u),
all i-fastest as in the reference's Ind_n
(src/main/amr/nmesh_amr_loops.h:279).
"""
import struct

import numpy as np

MAGIC = 0x44474D4E


def read_dump(path, with_r):
    """Return a dict of stacked arrays: pat[E], n[E,3], bbox[E,6], x[E,3,np],
    dXdx[E,9,np], sqrtgdiag[E,3,np], u[E,5,np] and r[E,5,np] if with_r;
    version-2 files add use_fv[E] and det_dXbdx[E,np]."""
    with open(path, "rb") as fp:
        buf = fp.read()
    magic, version, nelem = struct.unpack_from("<3i", buf, 0)
    if magic != MAGIC or version not in (1, 2):
        raise ValueError(f"{path}: not an nmgdump v1/v2 file")
    v2 = version == 2
    off = 12
    pats, ns, bboxes, xs, dxs, sgs, us, rs = [], [], [], [], [], [], [], []
    fvs, dets = [], []
    for _ in range(nelem):
        pat, n0, n1, n2 = struct.unpack_from("<4i", buf, off)
        off += 16
        if v2:
            fvs.append(struct.unpack_from("<i", buf, off)[0])
            off += 4
        bbox = np.frombuffer(buf, "<f8", 6, off)
        off += 48
        npt = n0 * n1 * n2
        g = 16 if v2 else 15          # geometry rows before u
        nblk = g + 5 + (5 if with_r else 0)
        blk = np.frombuffer(buf, "<f8", nblk * npt, off).reshape(nblk, npt)
        off += 8 * nblk * npt
        pats.append(pat)
        ns.append((n0, n1, n2))
        bboxes.append(bbox.copy())
        xs.append(blk[0:3].copy())
        dxs.append(blk[3:12].copy())
        sgs.append(blk[12:15].copy())
        if v2:
            dets.append(blk[15].copy())
        us.append(blk[g:g + 5].copy())
        if with_r:
            rs.append(blk[g + 5:g + 10].copy())
    if off != len(buf):
        raise ValueError(f"{path}: trailing bytes")
    out = dict(pat=np.array(pats, np.int32), n=np.array(ns, np.int32),
               bbox=np.array(bboxes), x=np.array(xs), dXdx=np.array(dxs),
               sqrtgdiag=np.array(sgs), u=np.array(us))
    if with_r:
        out["r"] = np.array(rs)
    if v2:
        out["use_fv"] = np.array(fvs, np.int32)
        out["det_dXbdx"] = np.array(dets)
    return out
