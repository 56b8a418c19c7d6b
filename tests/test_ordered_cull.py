"""CPU model of the ordered stage's occlusion tests: per tile (raster_kernels.cu may_pass_tile) and
per pixel (the candidate test of forward_tile, the same bound over one pixel's sample range).

A tile skips the in-order stage when none of its ordered entries may pass the depth test against
the tile's farthest prefix depth dmax.  The test restates the kernel's float32 arithmetic (the
depth plane's minimum over the triangle's bounding box clipped to the tile's sample positions,
less a margin of 2^-20 of the terms' magnitudes) and checks on random planes that whenever it
says "cannot pass", every sample position of the rectangle evaluates, in the per-sample order
the raster and ordered stages use ((z0 + dzdx (x - X0)) + dzdy (y - Y0), float32), to a depth
above dmax.
"""
import numpy as np

F = np.float32


def sample_depth(z0, dzdx, dzdy, X0, Y0, x, y):
    return F(F(z0 + F(dzdx * F(x - X0))) + F(dzdy * F(y - Y0)))


def may_pass(z0, dzdx, dzdy, X0, Y0, sx0, sx1, sy0, sy1, dmax):
    ax, bx = F(dzdx * F(sx0 - X0)), F(dzdx * F(sx1 - X0))
    ay, by = F(dzdy * F(sy0 - Y0)), F(dzdy * F(sy1 - Y0))
    zmin = F(F(z0 + min(ax, bx)) + min(ay, by))
    margin = F(F(F(abs(z0) + max(abs(ax), abs(bx))) + max(abs(ay), abs(by))) * F(2.0 ** -20))
    return not (F(zmin - margin) > dmax)


def test_culled_entries_fail_at_every_sample():
    rng = np.random.default_rng(3)
    culled = 0
    for _ in range(4000):
        X0, Y0 = (int(v) for v in rng.integers(-200000, 800000, 2))
        z0 = F(rng.uniform(0.0, 1.0))
        dzdx, dzdy = (F(v) for v in rng.normal(size=2) * 10.0 ** rng.uniform(-9, -4, 2))
        sx0 = int(rng.integers(0, 3840 * 256))
        sy0 = int(rng.integers(0, 2160 * 256))
        sx1, sy1 = sx0 + int(rng.integers(0, 16 * 256)), sy0 + int(rng.integers(0, 16 * 256))
        xs = np.unique(np.r_[np.linspace(sx0, sx1, 9).astype(np.int64), sx0, sx1])
        ys = np.unique(np.r_[np.linspace(sy0, sy1, 9).astype(np.int64), sy0, sy1])
        zs = [sample_depth(z0, dzdx, dzdy, X0, Y0, x, y) for x in xs for y in ys]
        zlow = min(zs)
        # dmax just below / at / just above the smallest sample depth, in float32 steps
        for dmax in (np.nextafter(zlow, F(-1)), zlow, np.nextafter(zlow, F(2)), F(zlow - F(1e-3))):
            if not may_pass(z0, dzdx, dzdy, X0, Y0, sx0, sx1, sy0, sy1, F(dmax)):
                culled += 1
                assert all(z > dmax for z in zs), (X0, Y0, z0, dzdx, dzdy, sx0, sx1, sy0, sy1, dmax)
    assert culled > 1000  # the test does cull


def test_pixel_boxes_culled_entries_fail_at_every_sample():
    """The per-pixel form: the sample range of one pixel (8x pattern bounds 16..240)."""
    rng = np.random.default_rng(5)
    culled = 0
    for _ in range(4000):
        X0, Y0 = (int(v) for v in rng.integers(-20000, 1000000, 2))
        z0 = F(rng.uniform(0.0, 1.0))
        dzdx, dzdy = (F(v) for v in rng.normal(size=2) * 10.0 ** rng.uniform(-9, -3, 2))
        px, py = int(rng.integers(0, 3840)), int(rng.integers(0, 2160))
        sx0, sx1, sy0, sy1 = px * 256 + 16, px * 256 + 240, py * 256 + 16, py * 256 + 240
        xs = np.arange(sx0, sx1 + 1, 16)
        ys = np.arange(sy0, sy1 + 1, 16)
        zs = [sample_depth(z0, dzdx, dzdy, X0, Y0, x, y) for x in xs for y in ys]
        zlow = min(zs)
        for dmax in (np.nextafter(zlow, F(-1)), zlow, np.nextafter(zlow, F(2)), F(zlow - F(1e-4))):
            if not may_pass(z0, dzdx, dzdy, X0, Y0, sx0, sx1, sy0, sy1, F(dmax)):
                culled += 1
                assert all(z > dmax for z in zs)
    assert culled > 1000
