"""The half-window split of VIEWSHED, checked on the CPU against the oracle.

`shed_half_kernel` (siting_gb300/csrc/viewshed.cu) sweeps an observer with
two CTAs: the upper one takes the 4roi+1 perimeter targets in rows <= the
observer's (perimeter order of siting.cpp:291-304), stages rows ox-roi..ox
and writes shed rows 0..roi; the lower one takes the other 4roi-1 targets,
stages rows ox..ox+roi and writes rows roi+1..2roi, dropping its marks on the
observer's row.  This module restates the kernel's ray partition and ray
sweep (siting.cpp:252-360, FP32 with IEEE division and round half away from
zero) and checks, per observer, that
* the two halves' rays are the 8roi perimeter rays, each once;
* every sample of a half lies in the rows that half stages;
* the lower half's marks on the observer's row are a subset of the upper
  half's (the reason they may be dropped);
* the upper half's rows 0..roi and the lower half's rows roi+1..2roi together
  equal the oracle's shed, bit for bit.
The restatement is test infrastructure; the GPU tests check the kernel itself.
"""
import numpy as np
import pytest

F32 = np.float32


def _round_away(v):
    v = float(v)
    r = int(np.floor(abs(v) + 0.5))
    return r if v >= 0 else -r


def half_ray(t, roi, half):
    """Perimeter index of ray t of a half (viewshed.cu: half_ray)."""
    if not half:
        return t + (0 if t <= roi else roi - 1 if t <= 2 * roi else 2 * roi - 1)
    return t + (roi + 1 if t < roi - 1 else 2 * roi + 1 if t < 2 * roi - 1 else 4 * roi + 1)


def sweep_half(dem, n, roi, oht, tht, ox, oy, half):
    """Marks (shed row, shed column) of one half's rays, and their perimeter indices."""
    side = 2 * roi
    xmin, ymin, xmax, ymax = ox - roi, oy - roi, ox + roi, oy + roi
    foalt, ftht = F32(int(dem[ox * n + oy]) + oht), F32(tht)
    marks, ips = set(), []
    for t in range(4 * roi - 1 if half else 4 * roi + 1):
        ip = half_ray(t, roi, half)
        ips.append(ip)
        if ip < side:
            tx, ty = xmin + ip, ymin
        elif ip < 2 * side:
            tx, ty = 1 + xmin - side + ip, ymax
        elif ip < 3 * side:
            tx, ty = xmin, 1 + ymin - 2 * side + ip
        else:
            tx, ty = xmax, ymin - 3 * side + ip
        dx, dy = tx - ox, ty - oy
        my = abs(dx) < abs(dy)
        dmaj, dmin = (dy, dx) if my else (dx, dy)
        d = 1 if dmaj > 0 else -1
        sl = F32(dmin) / F32(dmaj)
        sl = sl if d > 0 else -sl
        omaj, omin = (oy, ox) if my else (ox, oy)
        lo, hi = 0, min(dmaj * d, n - 1 - omaj if d > 0 else omaj)
        while lo < hi:  # last step inside the DEM and the roi circle
            mid = (lo + hi + 1) >> 1
            off = _round_away(F32(mid) * sl)
            if 0 <= omin + off < n and mid * mid + off * off <= roi * roi:
                lo = mid
            else:
                hi = mid - 1
        hs = F32(-99999.0)
        for k in range(1, lo + 1):
            fk = F32(k)
            off = _round_away(fk * sl)
            x, y = (ox + off, oy + d * k) if my else (ox + d * k, oy + off)
            assert (ox - roi <= x <= ox) if half == 0 else (ox <= x <= ox + roi), \
                f"half {half} ray {ip} step {k} leaves its rows"
            fe = F32(int(dem[x * n + y]))
            s = (fe - foalt) / fk
            hs = s if hs < s else hs
            if fe + ftht >= foalt + hs * fk:
                marks.add((x - xmin, y - ymin))
    return marks, ips


@pytest.mark.parametrize("roi,n,seed", [(1, 24, 1), (2, 30, 2), (3, 40, 3), (8, 50, 4), (14, 64, 5)])
def test_half_windows_partition_the_rays_and_give_the_oracle_shed(native, oracle, roi, n, seed):
    dem = native.fbm_dem(n, seed, octaves=6, range_max=3000)
    dem.reshape(n, n)[n // 3:n // 2, n // 4:n // 2] = 1200  # a plateau: ties along straight rays
    rng = np.random.default_rng(seed)
    obs = np.array(list(rng.choice(n * n, 6, replace=False)) +
                   [0, n - 1, n * n - 1, n * (n - 1), n // 2, (n // 2) * n,
                    (n // 3 + 1) * n + n // 3], np.int32)
    want = oracle.sheds(dem, n, roi, 20, 20, obs)
    nr = 2 * roi + 1
    nwpr = (nr + 63) // 64
    for i, ob in enumerate(obs):
        ox, oy = divmod(int(ob), n)
        upper, ips0 = sweep_half(dem, n, roi, 20, 20, ox, oy, 0)
        lower, ips1 = sweep_half(dem, n, roi, 20, 20, ox, oy, 1)
        assert sorted(ips0 + ips1) == list(range(8 * roi))
        upper.add((roi, roi))  # the observer's own cell (siting.cpp:279)
        assert {m for m in lower if m[0] == roi} <= {m for m in upper if m[0] == roi}
        got = np.zeros(nr * nwpr, np.uint64)
        for r, c in {m for m in upper if m[0] <= roi} | {m for m in lower if m[0] > roi}:
            got[r * nwpr + c // 64] |= np.uint64(1) << np.uint64(63 - c % 64)
        w = want[i * nr * nwpr:(i + 1) * nr * nwpr]
        assert np.array_equal(got, w), f"observer {ob}: {np.count_nonzero(got != w)} words differ"
