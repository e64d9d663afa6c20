"""AMOEBA topology set-up: local frames, multipole units, polarization groups
and the scaled-pair (exclusion) table consumed by the polarization kernels.

In Tinker9 this information comes from Fortran Tinker (kmpole, kpolar,
polargrp, attach) through module globals; the reference then turns it into
device tables in src/amoeba/epolar.cpp:88-510 (d/p/u scales) and
src/elec.cpp:54-140 (frames and multipoles).  This module restates that set-up
for the inputs this project needs, with the same semantics:

* multipole units: dipoles x bohr, quadrupoles x bohr^2 / 3 (Tinker kmpole);
* frame type from the signs of the axis types (Tinker kmpole): 0 -> None,
  z only -> Z-Only, z<0 or x<0 -> Bisector, x<0 and y<0 -> Z-Bisect,
  all < 0 -> 3-Fold, otherwise Z-then-X;
* pdamp = alpha^(1/6) (Tinker kpolar); Thole pair value min(thole_i, thole_k)
  (include/seq/damp.h:18-22);
* polarization group = bonded atoms whose types list each other on their
  `polarize` records; d and u scales by group distance (11, 12, 13, 14);
  p scales by bond distance (12..15), with the "intra" values when both atoms
  share a group; m scales by bond distance (12..15).

Scale table rows are (i, k) with i < k and columns (m, d, p, u); pairs whose
four scales are all one are omitted.
"""
from collections import deque

import numpy as np

from .units import BOHR

LF_NONE, LF_Z_ONLY, LF_Z_THEN_X, LF_BISECTOR, LF_Z_BISECT, LF_3_FOLD = 0, 1, 2, 3, 4, 5


def frame_kind(kz, kx, ky):
    """Tinker kmpole rule for the local-frame type from signed axis types."""
    kind = LF_Z_THEN_X
    if kz == 0:
        kind = LF_NONE
    if kz != 0 and kx == 0:
        kind = LF_Z_ONLY
    if kz < 0 or kx < 0:
        kind = LF_BISECTOR
    if kx < 0 and ky < 0:
        kind = LF_Z_BISECT
    if max(kz, kx, ky) < 0:
        kind = LF_3_FOLD
    return kind


def pole_from_record(values):
    """Parameter-file multipole (q; dx dy dz; qxx; qyx qyy; qzx qzy qzz) in
    e, e*bohr, e*bohr^2 -> MPL order [q, dx, dy, dz, qxx, qyy, qzz, qxy, qxz,
    qyz] in e, e*A, e*A^2 with the 1/3 quadrupole factor."""
    q = values[0]
    d = [v * BOHR for v in values[1:4]]
    f = BOHR * BOHR / 3.0
    qxx, qyx, qyy, qzx, qzy, qzz = [v * f for v in values[4:10]]
    return [q, d[0], d[1], d[2], qxx, qyy, qzz, qyx, qzx, qzy]


def bond_distance_lists(n, bonds, maxd=4):
    """Shortest bond-path separation up to maxd for every atom: dict i -> {k: d}."""
    adj = [[] for _ in range(n)]
    for i, k in bonds:
        adj[i].append(k)
        adj[k].append(i)
    sep = []
    for i in range(n):
        dist = {i: 0}
        dq = deque([i])
        while dq:
            a = dq.popleft()
            if dist[a] == maxd:
                continue
            for b in adj[a]:
                if b not in dist:
                    dist[b] = dist[a] + 1
                    dq.append(b)
        del dist[i]
        sep.append(dist)
    return adj, sep


def assign_frames(types, adj, records):
    """Pick z/x/y axis atoms for each site from its multipole records.

    records: type -> list of (kz, kx, ky, values).  z is searched among the
    atom's neighbours, x and y first among its neighbours and then among the
    z atom's neighbours, lowest index first.  Returns frames[n][4] = (zaxis,
    xaxis, yaxis 1-based signed, kind) and the local poles [n][10].
    """
    n = len(types)
    frames = np.zeros((n, 4), dtype=np.int32)
    poles = np.zeros((n, 10))
    for i in range(n):
        recs = records[types[i]]
        done = False
        for kz, kx, ky, vals in recs:
            kind = frame_kind(kz, kx, ky)
            if kind == LF_NONE:
                frames[i] = (0, 0, 0, LF_NONE)
                poles[i] = pole_from_record(vals)
                done = True
                break
            for z in sorted(adj[i]):
                if types[z] != abs(kz):
                    continue
                if kind == LF_Z_ONLY:
                    frames[i] = (z, 0, 0, kind)
                    poles[i] = pole_from_record(vals)
                    done = True
                    break
                xcand = [a for a in sorted(adj[i]) if a != z] + [a for a in sorted(adj[z]) if a != i]
                for x in xcand:
                    if types[x] != abs(kx):
                        continue
                    if ky == 0:
                        frames[i] = (z, x, 0, kind)
                        poles[i] = pole_from_record(vals)
                        done = True
                        break
                    ycand = [a for a in sorted(adj[i]) if a not in (z, x)] + [
                        a for a in sorted(adj[z]) if a not in (i, x)
                    ]
                    for y in ycand:
                        if types[y] == abs(ky):
                            ysign = -1 if ky < 0 and kind == LF_Z_THEN_X else 1
                            frames[i] = (z, x, ysign * (y + 1), kind)
                            poles[i] = pole_from_record(vals)
                            done = True
                            break
                    if done:
                        break
                if done:
                    break
            if done:
                break
        if not done:
            raise ValueError(f"no multipole frame found for atom {i} (type {types[i]})")
    return frames, poles


def polar_groups(types, bonds, group_types):
    """Union bonded atoms whose types list each other (either direction)."""
    n = len(types)
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for i, k in bonds:
        if types[k] in group_types.get(types[i], ()) or types[i] in group_types.get(types[k], ()):
            ri, rk = find(i), find(k)
            if ri != rk:
                parent[rk] = ri
    return np.array([find(i) for i in range(n)], dtype=np.int64)


def group_distances(n, bonds, grp, maxd=3):
    """Separation between atoms' groups in the group graph (0 = same group)."""
    gids = sorted(set(grp.tolist()))
    gadj = {g: set() for g in gids}
    for i, k in bonds:
        gi, gk = grp[i], grp[k]
        if gi != gk:
            gadj[gi].add(gk)
            gadj[gk].add(gi)
    gdist = {}
    for g in gids:
        dist = {g: 0}
        dq = deque([g])
        while dq:
            a = dq.popleft()
            if dist[a] == maxd:
                continue
            for b in gadj[a]:
                if b not in dist:
                    dist[b] = dist[a] + 1
                    dq.append(b)
        gdist[g] = dist
    members = {}
    for i, g in enumerate(grp.tolist()):
        members.setdefault(g, []).append(i)
    return gdist, members


DEFAULT_SCALES = {
    "mpole-12-scale": 0.0, "mpole-13-scale": 0.0, "mpole-14-scale": 0.4, "mpole-15-scale": 0.8,
    "polar-12-scale": 0.0, "polar-13-scale": 0.0, "polar-14-scale": 1.0, "polar-15-scale": 1.0,
    "polar-12-intra": 0.0, "polar-13-intra": 0.0, "polar-14-intra": 0.5, "polar-15-intra": 1.0,
    "direct-11-scale": 0.0, "direct-12-scale": 1.0, "direct-13-scale": 1.0, "direct-14-scale": 1.0,
    "mutual-11-scale": 1.0, "mutual-12-scale": 1.0, "mutual-13-scale": 1.0, "mutual-14-scale": 1.0,
}


def scale_table(n, bonds, grp, scales):
    """Rows (i, k, m, d, p, u) for every pair with a scale different from 1."""
    _, sep = bond_distance_lists(n, bonds, 4)
    gdist, members = group_distances(n, bonds, grp, 3)
    pairs = {}

    def row(i, k):
        key = (min(i, k), max(i, k))
        if key not in pairs:
            pairs[key] = [1.0, 1.0, 1.0, 1.0]
        return pairs[key]

    mkey = {1: "mpole-12-scale", 2: "mpole-13-scale", 3: "mpole-14-scale", 4: "mpole-15-scale"}
    pkey = {1: "polar-12-scale", 2: "polar-13-scale", 3: "polar-14-scale", 4: "polar-15-scale"}
    pikey = {1: "polar-12-intra", 2: "polar-13-intra", 3: "polar-14-intra", 4: "polar-15-intra"}
    dkey = {0: "direct-11-scale", 1: "direct-12-scale", 2: "direct-13-scale", 3: "direct-14-scale"}
    ukey = {0: "mutual-11-scale", 1: "mutual-12-scale", 2: "mutual-13-scale", 3: "mutual-14-scale"}
    for i in range(n):
        for k, d in sep[i].items():
            if k <= i:
                continue
            ms = scales[mkey[d]]
            ps = scales[pikey[d]] if grp[i] == grp[k] else scales[pkey[d]]
            if ms != 1.0:
                row(i, k)[0] = ms
            if ps != 1.0:
                row(i, k)[2] = ps
        for g, gd in gdist[grp[i]].items():
            ds, us = scales[dkey[gd]], scales[ukey[gd]]
            if ds == 1.0 and us == 1.0:
                continue
            for k in members[g]:
                if k <= i:
                    continue
                if ds != 1.0:
                    row(i, k)[1] = ds
                if us != 1.0:
                    row(i, k)[3] = us
    keys = sorted(k for k, v in pairs.items() if any(x != 1.0 for x in v))
    ik = np.array(keys, dtype=np.int32).reshape(-1, 2)
    sc = np.array([pairs[k] for k in keys], dtype=np.float64).reshape(-1, 4)
    return ik, sc
