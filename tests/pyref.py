"""Independent pure-Python restatement of the integration call for tiny cases.

Written separately from oracle/tsdf_oracle.cpp, with numpy float32 scalars
(IEEE single, round to nearest, no contraction), so the C++ oracle can be
checked against a second implementation of the same formulas
(tsdf_package/src/cuda/tsdf_handler.cu of ros_tsdf):

  center      :65-85    floor(x * (1/s)) / (1/s) + s/2
  segment     :112-133  p -/+ T * (p - s)/|p - s|, nearer end first
  traverse    :146-245  float DDA with the reference's tie rules, epsilon
                        termination and step-size abort
  distance    :562-573  +-|p - x|, negative when (p-s).(p-x) < 0
  weight      :579-581  1 / (|d| + 1)
  update      :648-654  W' = W + w; sdf = (W sdf + w d) / W'; W = min(W', max)
  publish     :749-825  blocks whose centre is within the publish radius,
                        voxels with weight != 0 at (i*vs + vs/2) + corner
  gc          :836-952  blocks beyond the gc radius freed, slots pushed

with the canonical orders the engine fixes: first-touch allocation, updates in
ascending point index, publish in ascending (slot, voxel), gc pushes in
ascending slot.  Loops are pure Python: use only for a few dozen points.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32


def derive(vs, T):
    vs, T = F(vs), F(T)
    bs = vs * F(8)
    t2 = T * F(2)
    vmax = int(F(math.ceil(t2 / vs)) * F(4))
    amax = int(F(math.ceil(t2 / bs)) * F(4))
    return dict(vs=vs, T=T, bs=bs, half_vs=vs / F(2), half_bs=bs / F(2), vmax=vmax, amax=amax, rmax=amax + 4,
                margin=amax + vmax // 8 + 2)


def center(x, s):
    scale = F(1) / F(s)
    f = F(np.floor(F(x) * scale))
    return f / scale + F(s) / F(2), int(f)


def sq3(a, b, c):
    return (a * a + b * b) + c * c


def segment(p, s, T):
    p = [F(v) for v in p]
    s = [F(v) for v in s]
    if not all(np.isfinite(v) for v in p + s):
        return None
    v = [p[i] - s[i] for i in range(3)]
    mag = F(np.sqrt(sq3(*v)))
    if not (mag > 0) or not np.isfinite(mag):
        return None
    n = [v[i] / mag for i in range(3)]
    a = [p[i] - F(T) * n[i] for i in range(3)]
    b = [p[i] + F(T) * n[i] for i in range(3)]
    if sq3(*[b[i] - s[i] for i in range(3)]) < sq3(*[a[i] - s[i] for i in range(3)]):
        a, b = b, a
    return a, b


def traverse(start, end, vs, cap):
    vs = F(vs)
    half = vs / F(2)
    eps = vs / F(4)
    vpe, vme = vs + eps, vs - eps
    u = start
    v = [end[i] - start[i] for i in range(3)]
    step = [vs if v[i] > 0 else F(-1) * vs for i in range(3)]
    sc = [center(start[i], vs)[0] for i in range(3)]
    with np.errstate(divide="ignore", invalid="ignore"):
        tm = [F(abs((sc[i] - half - u[i]) / v[i] if v[i] < 0 else (sc[i] + half - u[i]) / v[i])) for i in range(3)]
        td = [F(abs(vs / v[i])) for i in range(3)]
    cur = list(start)
    cc = [center(cur[i], vs) for i in range(3)]
    ec = [center(end[i], vs)[0] for i in range(3)]
    out = []
    overflow = False

    def eq():
        return all(abs(cc[i][0] - ec[i]) < eps for i in range(3))

    while not eq():
        if len(out) == cap:
            return out, True
        out.append((tuple(c[0] for c in cc), tuple(c[1] for c in cc)))
        tx, ty, tz = tm
        if tx < ty:
            ax = [0] if tx < tz else ([2] if tx > tz else [0, 2])
        elif tx > ty:
            ax = [1] if ty < tz else ([2] if ty > tz else [1, 2])
        else:
            ax = [2] if tz < tx else ([0, 1] if tz > tx else [0, 1, 2])
        for i in ax:
            cur[i] = cur[i] + step[i]
            tm[i] = tm[i] + td[i]
        prev = [c[0] for c in cc]
        cc = [center(cur[i], vs) for i in range(3)]
        d = [abs(prev[i] - cc[i][0]) for i in range(3)]
        if (d[0] < vme and d[1] < vme and d[2] < vme) or (d[0] > vpe or d[1] > vpe or d[2] > vpe):
            return out, overflow
    if len(out) == cap:
        return out, True
    out.append((tuple(c[0] for c in cc), tuple(c[1] for c in cc)))
    return out, overflow


def distance(x, p, s):
    a = [F(p[i]) - F(s[i]) for i in range(3)]
    b = [F(p[i]) - F(x[i]) for i in range(3)]
    mag = F(np.sqrt(sq3(*b)))
    dot = (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]
    return mag * F(-1) if dot < 0 else mag


def weight(d):
    return F(1) / (F(abs(d)) + F(1))


def apply(sdf, w, d, maxw):
    wt = weight(d)
    wd = wt * d
    nw = w + wt
    return (w * sdf + wd) / nw, min(nw, F(maxw))


class PyMap:
    def __init__(self, vs, T, maxw, pub_d2, gc_d2, heap_blocks):
        self.d = derive(vs, T)
        self.maxw, self.pub_d2, self.gc_d2 = F(maxw), F(pub_d2), F(gc_d2)
        self.cap = heap_blocks
        self.free = list(range(heap_blocks))
        self.bc = 0
        self.table = {}      # key -> slot
        self.slot_key = {}   # slot -> key
        self.vox = {}        # slot -> (512, 2) float32

    def block_center(self, key):
        bs = self.d["bs"]
        scale = F(1) / bs
        return [F(k) / scale + bs / F(2) for k in key]

    def in_range(self, pt):
        lim = F((1 << 20) - self.d["margin"])
        for x in pt:
            f = F(np.floor(F(x) * (F(1) / self.d["bs"])))
            if not (f > -lim and f < lim):
                return False
        return True

    def integrate(self, pts, origin):
        d = self.d
        org = [F(v) for v in origin]
        segs = []
        new = []
        for p in pts:
            sg = segment(p, org, d["T"])
            if sg is None or not self.in_range(sg[0]) or not self.in_range(sg[1]):
                segs.append(None)
                continue
            segs.append(sg)
            cells, _ = traverse(sg[0], sg[1], d["bs"], d["amax"])
            for _, key in cells:
                if key not in self.table and key not in new:
                    new.append(key)
        for key in new:
            if self.bc >= self.cap:
                continue
            slot = self.free[self.bc]
            self.bc += 1
            self.table[key] = slot
            self.slot_key[slot] = key
            self.vox[slot] = np.zeros((512, 2), np.float32)
        for p, sg in zip(pts, segs):
            if sg is None:
                continue
            cells, _ = traverse(sg[0], sg[1], d["vs"], d["vmax"])
            run, run_key = -1, None
            for x, _ in cells:
                bcen = [center(x[i], d["bs"]) for i in range(3)]
                key = tuple(b[1] for b in bcen)
                if key != run_key:
                    run += 1
                    run_key = key
                if run >= d["rmax"] or key not in self.table:
                    continue
                slot = self.table[key]
                bl = [bcen[i][0] - d["half_bs"] for i in range(3)]
                idx = [int(np.floor((F(x[i]) - bl[i]) / d["vs"])) for i in range(3)]
                if not all(0 <= v < 8 for v in idx):
                    continue
                local = idx[0] + 8 * idx[1] + 64 * idx[2]
                dist = distance(x, p, org)
                s0, w0 = self.vox[slot][local]
                self.vox[slot][local] = apply(F(s0), F(w0), dist, self.maxw)
        pub = []
        for slot in sorted(self.slot_key):
            c = self.block_center(self.slot_key[slot])
            if sq3(*[org[i] - c[i] for i in range(3)]) > self.pub_d2:
                continue
            bl = [c[i] - d["half_bs"] for i in range(3)]
            for l in range(512):
                s_, w_ = self.vox[slot][l]
                if w_ == 0:
                    continue
                ijk = (l & 7, (l >> 3) & 7, l >> 6)
                pos = [F(ijk[i]) * d["vs"] + d["half_vs"] + bl[i] for i in range(3)]
                pub.append((pos, (s_, w_)))
        for slot in sorted(list(self.slot_key)):
            c = self.block_center(self.slot_key[slot])
            if sq3(*[org[i] - c[i] for i in range(3)]) <= self.gc_d2:
                continue
            del self.table[self.slot_key[slot]]
            del self.slot_key[slot]
            self.bc -= 1
            self.free[self.bc] = slot
        if not pub:
            return np.zeros((0, 3), np.float32), np.zeros((0, 2), np.float32)
        return (np.array([p for p, _ in pub], np.float32), np.array([v for _, v in pub], np.float32))
