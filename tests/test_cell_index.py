"""The lidar's division-free shortcuts are exactly the reference's arithmetic.

1. Nearest cell. racer/sim.mojo:110-114 computes ix = floor((x - x0) / cell
   + 0.5) with a binary32 division and tests 0 <= ix < nx. The CUDA probe
   (sim.cu, cell_of) computes v = RN(x * r + c) in one fused multiply-add,
   with r = RN(1 / cell) and c = RN(-x0 * r); when both |v - rint(v)| lie
   below band = 0.5 - (5.001 M + 4.001 X + 16) * 2^-24 (M = max(nx, ny),
   X = max(|x0|, |y0|) / cell), it uses rint(v) with an integer bounds test,
   otherwise the division (whose own shortcut, cell_coord, is replayed too).
   The claim: on-map status and cell are always the reference's.
2. Division skip. The guarded march (sim.cu, march<.., true>: rays with a
   huge or non-finite origin height or a subnormal descent) evaluates
   fl / descent only when fl * RN(1 / descent) <= a * (1 + 2^-20); the claim:
   whenever it skips, RN(fl / descent) >= a, so min(a, fl / descent) = a.
3. The quotient of the unguarded march (sim.cu, quotient; also the ray's
   normalisation, div_by, and the obs value range / 10, range_obs): from y = RN(1 / b) and
   q0 = RN(a * y), two residual corrections q <- RN(q + RN(a - b q) y), each a
   pair of fused multiply-adds, give RN(a / b); the claim is checked on the
   march's operand ranges, on wide exponents and on quotients a hair from a
   rounding midpoint.
4. The rounding in the unguarded march's probe (sim.cu, lidar_cell): rint(v)
   as (v + 1.5 * 2^23) - 1.5 * 2^23 and the cell as the sum's bits less those
   of 1.5 * 2^23 (unsigned); the claims: exact for |v| < 2^22, and an index of
   at least 2^22 (off any map) for every larger, infinite or NaN v.
5. The count-free march (sim.cu, march<.., false, false>): where the host
   sets TrackDev.free_march, the loop tests tt < RANGE alone; the claim: the
   probe bound max_iters = ceil(RANGE / (0.5 cell)) + 2 can never end the
   march first there, and the host's test keeps the bound for tiny cells.
6. The lidar's cells (api.cu, upload_track; sim.cu, lidar_probe): the layer
   choice folded into a per-cell (c0, h0, c1, h1) gives probe()'s clearance
   and height for every drivability pattern, NaN clearances, ties and
   off-map border cells.
7. The march's cell index along the ray (sim.cu, lidar_cell): v = RN(tt *
   RN(dx r) + RN(ox r + cx)) in one fused multiply-add instead of the probe
   point px = RN(ox + RN(tt dx)); the claim: wherever |v - rint(v)| lies
   inside the wider band 0.5 - (7.001 M + 2.001 X + 3.001 RANGE / cell + 16)
   * 2^-24, on-map status and cell are the reference's for px.

All are replayed here in numpy binary32 (IEEE round-to-nearest, like the
GPU built with --fmad=false; the fused multiply-add exactly, through a
binary64 product and an exact two-sum) on random values and on adversarial
ones a few ulps either side of every cell boundary and of the band's edge.
"""
import numpy as np
import pytest

f32, f64 = np.float32, np.float64


def fma32(a, b, c):
    """RN32(a * b + c) without intermediate rounding, for binary32 arrays."""
    p = a.astype(f64) * b.astype(f64)  # exact: 48 significant bits at most
    s = p + c.astype(f64)
    bb = s - p
    err = (p - (s - bb)) + (c.astype(f64) - bb)  # p + c = s + err exactly
    with np.errstate(all="ignore"):
        f = s.astype(f32)
        lo = np.where(f.astype(f64) <= s, f, np.nextafter(f, f32(-np.inf)))
        hi = np.nextafter(lo, f32(np.inf))
        tie = s == (lo.astype(f64) + hi.astype(f64)) / 2  # s halfway between two binary32 values
    # off a halfway point err cannot move s across one; on it, err decides (ties to even if err == 0)
    return np.where(tie & (err > 0), hi, np.where(tie & (err < 0), lo, f)).astype(f32)


def band_delta(v0, cell, nmax):
    X = np.ceil(abs(float(v0)) / float(cell))
    return (5.001 * nmax + 4.001 * X + 16.0) * 2.0 ** -24


def exact_cell(v, v0, cell, n):
    f = np.floor((v - v0) / cell + f32(0.5))
    on = (f >= 0) & (f < f32(n))
    return on, np.where(on, f, -1)


def division_free_coord(v, v0, cell):
    """sim.cu cell_coord: the division only within (|u| + 1) * 2^-20 of an integer."""
    r = f32(1) / cell
    d = v - v0
    u = d * r + f32(0.5)
    fl = np.floor(u)
    g = u - fl
    delta = (np.abs(u) + f32(1)) * f32(9.5367431640625e-07)
    return np.where((g > delta) & (g < f32(1) - delta), fl, np.floor(d / cell + f32(0.5)))


def fast_cell(v, v0, cell, n, nmax):
    r = f32(1) / cell
    c = f32(-v0 * r)
    band = f32(0.5 - band_delta(v0, cell, nmax) * (1 + 2.0 ** -20))
    u = fma32(v, np.full_like(v, r), np.full_like(v, c))
    fl = np.rint(u)
    ok = np.abs(u - fl) < band
    with np.errstate(invalid="ignore"):
        i = np.clip(np.nan_to_num(fl, nan=0, posinf=2**31 - 1, neginf=-2**31), -2**31, 2**31 - 1).astype(np.int64)
    on_fast = (i >= 0) & (i < n)
    fc = division_free_coord(v, v0, cell)
    on_slow = (fc >= 0) & (fc < f32(n))
    on = np.where(ok, on_fast, on_slow)
    idx = np.where(ok, np.where(on_fast, i.astype(f32), -1), np.where(on_slow, fc, -1))
    return on, idx, ok


@pytest.mark.parametrize("cell,n,nmax", [(0.025, 721, 721), (0.025, 441, 721), (0.05, 2048, 2048),
                                         (0.05, 281, 281), (0.0123, 900, 1400), (0.07, 100, 3000)])
def test_fast_cell_index_is_exact(cell, n, nmax):
    cell = f32(cell)
    rng = np.random.default_rng(int(cell * 1e4) + n)
    for v0 in (f32(-8.9999361), f32(-5.4998164), f32(-1), f32(3.3), f32(-52.1)):
        ks = np.arange(-60, n + 60)
        base = (v0 + (ks.astype(f32) + f32(0.5)) * cell).astype(f32)
        adv = [base]
        up, down = base.copy(), base.copy()
        for _ in range(40):
            up = np.nextafter(up, f32(np.inf))
            down = np.nextafter(down, f32(-np.inf))
            adv += [up, down]
        # points whose u' lands just inside and outside the band edge
        edge = f32(band_delta(v0, cell, nmax))
        for frac in (edge, -edge):
            target = (ks.astype(np.float64) + frac.astype(np.float64) * np.array([[0.5], [1.0], [1.5], [2.0]]))
            adv += list((v0 + (target - 0.5) * np.float64(cell)).astype(f32))
        span = float(n) * float(cell)
        uniform = rng.uniform(float(v0) - 0.3 * span, float(v0) + 1.3 * span, 400000).astype(f32)
        far = np.array([1e9, -1e9, 3e38, -3e38, np.inf, -np.inf, np.nan], f32)
        vs = np.concatenate(adv + [uniform, far]).astype(f32)
        with np.errstate(all="ignore"):
            on_ex, idx_ex = exact_cell(vs, v0, cell, n)
            on, idx, ok = fast_cell(vs, v0, cell, n, nmax)
        assert np.array_equal(on, on_ex)
        assert np.array_equal(idx[on], idx_ex[on])
        # the band is narrow: almost every uniformly placed lookup skips the division
        assert ok[len(vs) - len(far) - len(uniform):len(vs) - len(far)].mean() > 0.99


def test_division_skip_is_exact():
    rng = np.random.default_rng(0)
    n = 2_000_000
    a = (rng.uniform(0.0125, 3, n)).astype(f32)
    descent = np.concatenate([rng.uniform(1e-4, 2, n // 2), 10 ** rng.uniform(-6, 1, n - n // 2)]).astype(f32)
    # floors near the point where the two terms cross, plus random ones
    fl = np.where(rng.random(n) < 0.5, a * descent * (1 + rng.normal(0, 1e-6, n)).astype(f32),
                  rng.uniform(0, 2, n)).astype(f32)
    fl = np.abs(fl).astype(f32)
    inv = f32(1) / descent
    skip = (fl * inv) > (a * f32(1.00000095))
    q = fl / descent
    assert np.all(q[skip] >= a[skip])
    assert skip.any() and (~skip).any()


def test_quotient_by_residual_corrections_is_ieee_division():
    rng = np.random.default_rng(3)
    bad = total = 0
    for kind in range(6):
        n = 500_000
        if kind in (0, 3):  # the march: floors up to 20 m, descents 1e-4 .. 5
            a = rng.uniform(0, 20, n).astype(f32)
            b = (10 ** rng.uniform(-4, 0.7, n)).astype(f32)
        elif kind == 1:  # wide exponents
            a = (10 ** rng.uniform(-8, 8, n)).astype(f32)
            b = (10 ** rng.uniform(-8, 8, n)).astype(f32)
        elif kind in (2, 4):  # a / b within an ulp's fraction of a rounding midpoint
            q = (10 ** rng.uniform(-3, 2, n)).astype(f32)
            mid = (q.astype(f64) + np.nextafter(q, f32(np.inf)).astype(f64)) / 2
            b = (10 ** rng.uniform(-3, 1, n)).astype(f32)
            a = (mid * b.astype(f64)).astype(f32)
        else:  # divisor significands near 2 (the largest reciprocal error)
            b = ((1.9999 + rng.uniform(0, 1e-4, n)) * 2.0 ** rng.integers(-10, 4, n)).astype(f32)
            a = rng.uniform(0, 20, n).astype(f32)
        with np.errstate(all="ignore"):
            y = f32(1) / b
            q = a * y
            for _ in range(2):
                q = fma32(fma32(-q, b, a), y, q)
            ref = a / b
        ok = np.isfinite(ref) & (ref > 0)
        bad += int(np.sum(q[ok] != ref[ok]))
        total += int(ok.sum())
    assert total > 2_900_000 and bad == 0


def test_ray_normalisation_by_residual_corrections_is_ieee_division():
    """sim.cu div_by: the ray's components (either sign, zeros of either sign, magnitudes down to
    1e-20) over norms from 0.9 to 4, against IEEE division, signs of zero included."""
    rng = np.random.default_rng(11)
    n = 1_000_000
    a = (rng.choice([-1, 1], n) * 10 ** rng.uniform(-20, 0.3, n)).astype(f32)
    a[:1000] = f32(0)
    a[1000:2000] = f32(-0.0)
    b = rng.uniform(0.9, 4.0, n).astype(f32)
    with np.errstate(all="ignore"):
        y = f32(1) / b
        q = a * y
        for _ in range(2):
            q = fma32(fma32(-q, b, a), y, q)
        q = np.where(a == 0, a, q)
        ref = a / b
    assert np.array_equal(q, ref) and np.array_equal(np.signbit(q), np.signbit(ref))


def test_range_over_ten_by_residual_corrections_is_ieee_division():
    """sim.cu range_obs: RN(range / 10) as quotient(range, 10, 0.1f, range * 0.1f) for ranges from
    2^-60 up. With a fixed divisor every step of the corrections scales exactly with the dividend's
    power of two while no intermediate is subnormal (true from 2^-60), so one binade checked at every
    binary32 value covers every binade; the ranges' own [8, 10] and the lowest binade are checked too."""
    def corrected(a):
        with np.errstate(all="ignore"):
            ten, y = np.full_like(a, f32(10)), np.full_like(a, f32(0.1))
            q = a * y
            for _ in range(2):
                q = fma32(fma32(-q, ten, a), y, q)
        return q
    binades = [np.arange(0x3F800000, 0x40000000, dtype=np.uint32),  # [1, 2): every value
               np.arange(0x41000000, 0x41200001, dtype=np.uint32),  # [8, 10]
               np.arange(0x21800000, 0x21800000 + (1 << 20), dtype=np.uint32)]  # from 2^-60
    for bits in binades:
        for chunk in np.array_split(bits, 8):
            a = chunk.view(f32)
            assert np.array_equal(corrected(a), a / f32(10))


def test_magic_rounding_and_off_map_index():
    rng = np.random.default_rng(11)
    v = np.concatenate([rng.uniform(-3e6, 3e6, 1_000_000), rng.uniform(-5e7, 5e7, 500_000),
                        rng.standard_normal(500_000) * 1e3, rng.uniform(-1, 1, 200_000) + 0.5,
                        np.array([4194303.5, 4194304, -4194304, -4194303.5, 8388608, -8388608, 12582912, -12582912,
                                  1e30, -1e30, 3.4e38, -3.4e38, np.inf, -np.inf, np.nan])]).astype(f32)
    magic = f32(12582912.0)
    with np.errstate(all="ignore"):
        m = (v + magic).astype(f32)
        r = (m - magic).astype(f32)
        ix = (m.view(np.uint32).astype(np.int64) - 0x4B400000) & 0xFFFFFFFF
    small = np.abs(v) < f32(4194304)
    assert np.array_equal(r[small], np.rint(v[small]))
    assert np.array_equal(ix[small], np.rint(v[small]).astype(np.int64) & 0xFFFFFFFF)
    assert np.all(ix[~small] >= 4194304)


def test_march_reaches_range_before_the_probe_bound():
    """Every probe the march continues from adds a step >= m = 0.5 cell and RN(tt + step) >=
    (tt + m)(1 - 2^-24), so after k probes tt >= m k (1 - 2^-24)^k; where that reaches RANGE at
    k = max_iters (the host's test), `tt < RANGE` ends the loop no later than the bound would."""
    RANGE = f32(10)

    def free_march(cell):
        m = f32(0.5) * f32(cell)
        k = int(np.ceil(RANGE / m)) + 2
        return m, k, float(m) * k * (1.0 - 2.0 ** -24) ** k >= 10.0 * (1.0 + 1e-9)

    for cell in (0.025, 0.05, 0.0123, 0.1, 0.5, 0.004):
        m, k, free = free_march(cell)
        assert free
        tt, probes = f32(0), 0
        while tt < RANGE:  # the slowest march: every step exactly m
            tt = f32(tt + m)
            probes += 1
        assert probes < k
    assert not free_march(1e-4)[2]  # tiny cells keep the counted loop


def test_lidar_cells_choose_the_probes_layer():
    rng = np.random.default_rng(5)
    n = 400_000
    vals = np.array([-1.0, 0.0, -0.0, -0.5, np.nan, 1e-30, 0.3, 2.0], f32)
    c0 = np.where(rng.random(n) < 0.5, rng.choice(vals, n), rng.uniform(0.01, 3, n)).astype(f32)
    c1 = np.where(rng.random(n) < 0.5, rng.choice(vals, n), rng.uniform(0.01, 3, n)).astype(f32)
    h0 = rng.uniform(-2, 2, n).astype(f32)
    h1 = np.where(rng.random(n) < 0.2, h0, rng.uniform(-2, 4, n)).astype(f32)
    z = np.where(rng.random(n) < 0.1, (h0 + h1) / f32(2), rng.uniform(-3, 5, n)).astype(f32)
    z[:1000] = rng.uniform(-1e20, 1e20, 1000).astype(f32)
    # probe<2, false> (sim.cu): layer 0 if drivable, layer 1 if drivable and strictly nearer
    with np.errstate(invalid="ignore"):
        d0, d1 = c0 > 0, c1 > 0
        gap = np.where(d0, np.abs(h0 - z), f32(1e30))
        take1 = d1 & (np.abs(h1 - z) < gap)
    ref_c = np.where(take1, c1, np.where(d0, c0, f32(-1)))
    ref_h = np.where(take1, h1, h0)
    # the packed cell (upload_track) and lidar_probe's choice
    both = d0 & d1
    a = np.where(both | d0, c0, np.where(d1, c1, f32(-1)))
    b = np.where(both | d0, h0, np.where(d1, h1, h0))
    c = np.where(both, c1, f32(-1))
    d = np.where(both, h1, f32(np.nan))
    with np.errstate(invalid="ignore"):
        up = np.abs(d - z) < np.abs(b - z)
    assert np.array_equal(np.where(up, c, a), ref_c, equal_nan=True)
    assert np.array_equal(np.where(up, d, b), ref_h)
    # a border cell (-1, -1, -1, NaN) reads as off the map: clearance -1, height -1
    with np.errstate(invalid="ignore"):
        assert not (abs(f32(np.nan) - z) < abs(f32(-1) - z)).any()


def mband(x0, y0, cell, nmax):
    X = np.ceil(max(abs(float(x0)), abs(float(y0))) / float(cell))
    d = (7.001 * nmax + 2.001 * X + 3.001 * 10.0 / float(cell) + 16.0) * 2.0 ** -24
    return f32(0.5 - d * (1 + 2.0 ** -20))


@pytest.mark.parametrize("x0,cell,n,nmax", [(-8.9999361, 0.025, 721, 721), (-5.4998164, 0.025, 441, 721),
                                            (-51.2, 0.05, 2048, 2048), (3.3, 0.0123, 900, 1400),
                                            (-7.9985256, 0.025, 641, 641)])
def test_march_cell_index_along_the_ray_is_exact(x0, cell, n, nmax):
    x0, cell = f32(x0), f32(cell)
    rng = np.random.default_rng(n)
    r = f32(1) / cell
    c = f32(-x0 * r)
    band = mband(x0, x0, cell, nmax)
    span = float(n) * float(cell)
    m = 300_000
    ox = rng.uniform(float(x0) - 2, float(x0) + span + 2, m).astype(f32)
    dx = np.cos(rng.uniform(0, np.pi, m)).astype(f32)
    dx[:1000] = f32(1)
    dx[1000:2000] = f32(-1)
    # tt that puts px on a cell boundary of the reference (px = x0 + (k - 0.5) cell), then its neighbours
    k = rng.integers(-3, n + 3, m)
    with np.errstate(all="ignore"):
        t0 = ((x0.astype(f64) + (k - 0.5) * f64(cell)) - ox.astype(f64)) / dx.astype(f64)
    t0 = np.where(np.isfinite(t0) & (t0 >= 0) & (t0 < 10), t0, rng.uniform(0, 10, m)).astype(f32)
    tts, oxs, dxs = [t0], [ox], [dx]
    up, down = t0.copy(), t0.copy()
    for _ in range(24):
        up, down = np.nextafter(up, f32(np.inf)), np.nextafter(down, f32(-np.inf))
        tts += [up, down]
        oxs += [ox, ox]
        dxs += [dx, dx]
    tts.append(rng.uniform(0, 10, m).astype(f32))
    oxs.append(ox)
    dxs.append(dx)
    tt, ox, dx = (np.concatenate(a).astype(f32) for a in (tts, oxs, dxs))
    keep = (tt >= 0) & (tt < f32(10))
    tt, ox, dx = tt[keep], ox[keep], dx[keep]
    with np.errstate(all="ignore"):
        px = (ox + (tt * dx).astype(f32)).astype(f32)
        on_ex, idx_ex = exact_cell(px, x0, cell, n)
        v = fma32(tt, (dx * r).astype(f32), fma32(ox, np.full_like(ox, r), np.full_like(ox, c)))
        rv = np.rint(v)
        ok = np.abs(v - rv) < band
    on = (rv >= 0) & (rv < n)
    assert np.array_equal(on[ok], on_ex[ok])
    assert np.array_equal(rv[ok & on], idx_ex[ok & on])
    assert (~ok).sum() > 0 and ok[-m:].mean() > 0.99
