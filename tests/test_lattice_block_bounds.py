"""CPU check of the bound the lattice sweep's block walks rely on
(worldline-flux-tube-lattice_gb300/csrc/wl_sweep.cuh, sweep_tile_lat): for a
block of 32 staged points, the box of the points its segments touch, mapped
through the same fma as the points and measured from an image centre in
FP32, bounds every Simpson node of those segments from below, so that

  box x > 19   ->  every node x > 18  (reciprocal-only walk),
  box x > 0.55 ->  every node x >= 0.5 (large-x form alone),

with the node values computed in FP32 as lat_seg2 computes them.  Seeded
oracle loops, centres over the unit cell, proper times over the lattice
configuration's range, the kernel's image selection (|R| <= 12 a and within
sqrt(18) lambda of the loop's scaled bounding box)."""
import numpy as np

from oracle import oracle as O

f32 = np.float32
SUB, CHUNK = 32, 256


def fl(v):
    return np.asarray(v, dtype=np.float64).astype(f32)


def fma(a, b, c):
    # product of two floats exact in FP64, one rounding to FP32 (a double
    # rounding differs from a fused fma by at most an ulp: far inside margins)
    return fl(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def segments_of_block(c0, b, ppl):
    """(i, j) point pairs of the group walk over block b of the chunk at c0."""
    qa = 1 if c0 == 0 else c0 // 4
    q0 = max(qa, (c0 + b * SUB) // 4)
    q1 = min((c0 + CHUNK) // 4, (c0 + (b + 1) * SUB) // 4, ppl // 4)
    out = []
    for q in range(q0, q1):
        out += [(4 * q - 4, 4 * q), (4 * q - 1, 4 * q + 1), (4 * q - 2, 4 * q + 2),
                (4 * q + 1, 4 * q + 3)]
    return np.array(out, dtype=np.int64).reshape(-1, 2)


def node_x(uix, uiy, ujx, ujy, il2):
    """x at the five Simpson nodes, FP32 as lat_seg2 (shape [..., 5])."""
    dx, dy = fl(ujx - uix), fl(ujy - uiy)
    as_ = fl(fma(uix, uix, fl(uiy * uiy)) * il2)
    bs = fl(fma(uix, dx, fl(uiy * dy)) * il2)
    cs = fl(fma(dx, dx, fl(dy * dy)) * il2)
    xs = [as_]
    for t in (0.25, 0.5, 0.75):
        xs.append(fma(fma(cs, f32(0.5 * t), bs), f32(2.0 * t), as_))
    xs.append(fl(fma(bs, f32(2.0), as_) + cs))
    return np.stack(xs, axis=-1)


def test_block_box_bounds_every_node():
    rng = np.random.default_rng(11)
    ppl = 512
    loops = O.vloops(9, 6, ppl)
    checked = {"far": 0, "mid": 0}
    for a in (2.0, 5.0, 10.0):
        for l2 in (1.0, 0.25):
            lam, il2 = np.sqrt(l2), f32(1.0 / l2)
            rcut, lim = 4.242640687119285 * lam, 12
            for _ in range(4):
                cx, cy = fl(rng.uniform(0, a)), fl(rng.uniform(0, a))
                s = fl(np.sqrt(np.exp(rng.uniform(np.log(1e-2), np.log(1e2)))))
                for L in loops:
                    w = L[:, :2].astype(f32)
                    bb = (w[:, 0].min(), w[:, 0].max(), w[:, 1].min(), w[:, 1].max())
                    m0 = max(-lim, int(np.ceil((s * bb[0] + cx - rcut) / a)))
                    m1 = min(lim, int(np.floor((s * bb[1] + cx + rcut) / a)))
                    n0 = max(-lim, int(np.ceil((s * bb[2] + cy - rcut) / a)))
                    n1 = min(lim, int(np.floor((s * bb[3] + cy + rcut) / a)))
                    mm, nn = np.meshgrid(np.arange(m0, m1 + 1), np.arange(n0, n1 + 1),
                                         indexing="ij")
                    ok = mm ** 2 + nn ** 2 <= 144
                    if not ok.any():
                        continue
                    crx = fma(-mm[ok].astype(f32), f32(a), cx)[:, None]   # [img, 1]
                    cry = fma(-nn[ok].astype(f32), f32(a), cy)[:, None]
                    ux, uy = fma(s, w[None, :, 0], crx), fma(s, w[None, :, 1], cry)
                    for c0 in range(0, ppl, CHUNK):
                        for b in range(CHUNK // SUB):
                            seg = segments_of_block(c0, b, ppl)
                            if len(seg) == 0:
                                continue
                            lo = max(c0 + b * SUB - 4, c0 if c0 == 0 else c0 - 4)
                            hi = min(c0 + (b + 1) * SUB, ppl)
                            bx0, bx1 = w[lo:hi, 0].min(), w[lo:hi, 0].max()
                            by0, by1 = w[lo:hi, 1].min(), w[lo:hi, 1].max()
                            lx, hx = fma(s, bx0, crx[:, 0]), fma(s, bx1, crx[:, 0])
                            ly, hy = fma(s, by0, cry[:, 0]), fma(s, by1, cry[:, 0])
                            ex = np.maximum(np.maximum(lx, -hx), f32(0))
                            ey = np.maximum(np.maximum(ly, -hy), f32(0))
                            xb = fl(fma(ex, ex, fl(ey * ey)) * il2)            # [img]
                            x = node_x(ux[:, seg[:, 0]], uy[:, seg[:, 0]],
                                       ux[:, seg[:, 1]], uy[:, seg[:, 1]], il2)
                            xmin = x.reshape(len(xb), -1).min(axis=1)
                            far, mid = xb > f32(19.0), xb > f32(0.55)
                            assert np.all(xmin[far] > 18.0), (a, l2, c0, b)
                            assert np.all(xmin[mid] >= 0.5), (a, l2, c0, b)
                            checked["far"] += int(far.sum())
                            checked["mid"] += int((mid & ~far).sum())
    # the bound was exercised on both kinds of blocks
    assert checked["far"] > 1000 and checked["mid"] > 1000, checked
