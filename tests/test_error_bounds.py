"""The float pre-tests of the periodogram count and of the ANIMATE renderer, restated in numpy on
the CPU, against the FP64 decisions they stand in for.

Both kernels decide most cases in float and hand the rest to the reference's FP64 expressions;
their frames and counts equal the oracle's byte for byte only if the float decision is never
taken where it could differ from the FP64 one.  These tests replay the float arithmetic (float32
numpy, one rounding per operation; fused multiply-adds emulated through float64, exact for a
float product) on millions of cases, many of them placed on the decision boundary, and check
that every case the float test settles is settled as FP64 settles it."""
import numpy as np

U = np.float32(2.0 ** -24)
f32 = np.float32


def fmaf(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


# ---------------------------------------------------------------- periodogram

def periodogram_fast(dt, fr):
    """(decided, counts) of the count kernel's fast test (csrc/periodogram.cu test_interval)."""
    dth = dt.astype(np.float32)
    fh = fr.astype(np.float32)
    kround = f32(12582912.0)
    y = fmaf(dth, fh, np.full_like(dth, kround))
    r = (y - kround).astype(np.float32)
    d = fmaf(dth, fh, -r)
    a = (np.abs(d) - f32(0.1)).astype(np.float32)
    thr = (fh * f32(2.4e-7)).astype(np.float32)
    bound = fmaf(dth, thr, np.full_like(dth, f32(1e-7)))
    return np.abs(a) > bound, a < 0


def periodogram_exact(dt, fr):
    """misc.c:145: |dt/dt1 - int(dt/dt1 + 0.5)| < 0.1 with dt1 = 1/fr."""
    dt1 = 1.0 / fr
    x = dt / dt1
    return np.abs(x - np.trunc(x + 0.5)) < 0.1


def test_periodogram_fast_test_agrees_with_fp64():
    rng = np.random.default_rng(1)
    n = 2_000_000
    fr = 1 / (80 / 24) + rng.integers(0, 10000, n) / 9999 * (24 - 1 / (80 / 24))
    dt = rng.uniform(1e-3, 60.0, n)
    # half of the cases on the threshold: dt/dt1 within 1e-6 of k +- 0.1
    k = np.floor(dt * fr)
    edge = k + rng.choice([-0.1, 0.1], n) + rng.uniform(-1e-6, 1e-6, n)
    dt[: n // 2] = np.maximum(edge[: n // 2], 0.05) / fr[: n // 2]
    decided, fast = periodogram_fast(dt, fr)
    exact = periodogram_exact(dt, fr)
    assert np.array_equal(fast[decided], exact[decided])
    assert decided[n // 2:].mean() > 0.999          # random intervals: nearly all settled in float
    assert decided[: n // 2].mean() < 0.5          # boundary cases: mostly left to FP64


# ---------------------------------------------------------------- renderer

def random_geometry(rng, n):
    out = np.zeros((n, 20))
    for i in range(n):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        bx, cx, ax = q[:, 0], q[:, 1], np.cross(q[:, 0], q[:, 1])
        c = 10 ** rng.uniform(-2, 0)
        b = c + rng.uniform(0, 1) * (1 - c)
        E = rng.standard_normal(3)
        E /= np.linalg.norm(E)
        out[i, 0:2] = (b, c)
        out[i, 2:5] = E
        out[i, 5:8] = (bx @ E, cx @ E, ax @ E)
        out[i, 11:14], out[i, 14:17], out[i, 17:20] = bx, cx, ax
    return out


def render_screen(g, cz, cy, S):
    """screen_background (csrc/animate.cu) for corners (cz, cy) of one frame, float32, with the
    running error bound; True where the corner is certainly background."""
    Ex, Ey, Ez = g[2], g[3], g[4]
    scale = 1.0 / np.sqrt(Ex * Ex + Ez * Ez)
    Y1 = [f32(-Ex * Ey * scale), f32((Ex * Ex + Ez * Ez) * scale), f32(-Ey * Ez * scale)]
    Z1x, Z1z = f32(-Ez * scale), f32(Ex * scale)
    b, c = g[0], g[1]
    bb, cc = b * b, c * c
    A = (g[5] * g[5] / bb + g[6] * g[6] / cc) + g[7] * g[7]
    ax = [f32(v) for v in g[11:20]]
    Ep = [f32(g[5]), f32(g[6]), f32(g[7])]
    ibb, icc, Af = f32(1.0 / bb), f32(1.0 / cc), f32(A)
    fS = f32(S)
    z1 = ((f32(2.4) * (cz - S // 2).astype(np.float32)) / fS).astype(np.float32)
    y1 = ((f32(2.4) * (cy - S // 2).astype(np.float32)) / fS).astype(np.float32)
    ez1, ey1 = f32(4) * U * np.abs(z1), f32(4) * U * np.abs(y1)

    def pm(x, ex, y, ey):
        z = (x * y).astype(np.float32)
        return z, (np.abs(x) * ey + np.abs(y) * ex + U * np.abs(z)).astype(np.float32)

    def ps(x, ex, y, ey):
        z = (x + y).astype(np.float32)
        return z, (ex + ey + U * np.abs(z)).astype(np.float32)

    yx = pm(y1, ey1, Y1[0], U * abs(Y1[0]))
    zx = pm(z1, ez1, Z1x, U * abs(Z1x))
    px = ps(*yx, *zx)
    py = pm(y1, ey1, Y1[1], U * abs(Y1[1]))
    yz = pm(y1, ey1, Y1[2], U * abs(Y1[2]))
    zz = pm(z1, ez1, Z1z, U * abs(Z1z))
    pz = ps(*yz, *zz)
    pbca = []
    for r in range(3):
        a0, a1, a2 = ax[3 * r], ax[3 * r + 1], ax[3 * r + 2]
        t0 = pm(a0, U * abs(a0), *px)
        t1 = pm(a1, U * abs(a1), *py)
        t2 = pm(a2, U * abs(a2), *pz)
        pbca.append(ps(*ps(*t0, *t1), *t2))
    (pb, epb), (pc, epc), (pa, epa) = pbca
    tb = pm(*pm(pb, epb, Ep[0], U * abs(Ep[0])), ibb, U * ibb)
    tc = pm(*pm(pc, epc, Ep[1], U * abs(Ep[1])), icc, U * icc)
    ta = pm(pa, epa, Ep[2], U * abs(Ep[2]))
    s2 = ps(*ps(*tb, *tc), *ta)
    B, eB = f32(2) * s2[0], f32(2) * s2[1]
    Babs = f32(2) * (np.abs(tb[0]) + np.abs(tc[0]) + np.abs(ta[0]))
    qb = pm(*pm(pb, epb, pb, epb), ibb, U * ibb)
    qc = pm(*pm(pc, epc, pc, epc), icc, U * icc)
    qa = pm(pa, epa, pa, epa)
    r2 = ps(*ps(*qb, *qc), *qa)
    C, eC = ps(r2[0], r2[1], f32(-1), f32(0))
    Cabs = qb[0] + qc[0] + qa[0] + f32(1)
    BB, eBB = pm(B, eB, B, eB)
    AC, eAC = pm(Af, U * abs(Af), C, eC)
    D, eD = ps(BB, eBB, f32(-4) * AC, f32(4) * eAC)
    M = Babs * Babs + f32(4) * abs(Af) * Cabs
    return (D + f32(2) * eD + f32(1e-12) * M) < 0


def render_hits(g, cz, cy, S):
    """The reference's FP64 discriminant test D >= 0 (cuda.c:2433-2462), in its operation order."""
    Ex, Ey, Ez = g[2], g[3], g[4]
    scale = 1.0 / np.sqrt(Ex * Ex + Ez * Ez)
    Z1x, Z1y, Z1z = -Ez * scale, 0.0, Ex * scale
    Y1x, Y1y, Y1z = -Ex * Ey * scale, (Ex * Ex + Ez * Ez) * scale, -Ey * Ez * scale
    z1 = 2.4 * (cz - S // 2).astype(np.float64) / S
    y1 = 2.4 * (cy - S // 2).astype(np.float64) / S
    p_x, p_y, p_z = y1 * Y1x + z1 * Z1x, y1 * Y1y + z1 * Z1y, y1 * Y1z + z1 * Z1z
    p_b = g[11] * p_x + g[12] * p_y + g[13] * p_z
    p_c = g[14] * p_x + g[15] * p_y + g[16] * p_z
    p_a = g[17] * p_x + g[18] * p_y + g[19] * p_z
    b, c, Epb, Epc, Epa = g[0], g[1], g[5], g[6], g[7]
    A = Epb * Epb / (b * b) + Epc * Epc / (c * c) + Epa * Epa
    B = 2.0 * (p_b * Epb / (b * b) + p_c * Epc / (c * c) + p_a * Epa)
    C = p_b * p_b / (b * b) + p_c * p_c / (c * c) + p_a * p_a - 1.0
    return B * B - 4.0 * A * C >= 0.0


def test_render_screen_never_settles_a_hit():
    rng = np.random.default_rng(2)
    S = 1080
    settled, total = 0, 0
    for g in random_geometry(rng, 24):
        cz = rng.integers(0, S + 1, 60_000)
        cy = rng.integers(0, S + 1, 60_000)
        screen = render_screen(g, cz, cy, S)
        hits = render_hits(g, cz, cy, S)
        assert not np.any(screen & hits)
        settled += int(screen.sum())
        total += int((~hits).sum())
    assert settled > 0.95 * total    # the background is almost all settled in float


def test_render_screen_on_the_silhouette():
    """Corners next to the silhouette (where D changes sign along a row), over many frame sizes:
    the pre-test settles none of the hits, and leaves the closest misses to FP64."""
    rng = np.random.default_rng(3)
    checked = 0
    for g in random_geometry(rng, 16):
        for S in rng.integers(100, 2000, 6) * 2:
            rows = rng.integers(0, S + 1, 40)
            cz = np.repeat(rows, S + 1)
            cy = np.tile(np.arange(S + 1), rows.size)
            hits = render_hits(g, cz, cy, S).reshape(rows.size, S + 1)
            edge = np.zeros_like(hits)
            change = hits[:, 1:] != hits[:, :-1]
            edge[:, 1:] |= change
            edge[:, :-1] |= change
            if not edge.any():
                continue
            z, y = cz.reshape(hits.shape)[edge], cy.reshape(hits.shape)[edge]
            screen = render_screen(g, z, y, int(S))
            assert not np.any(screen & hits[edge])
            checked += int(edge.sum())
    assert checked > 1000
