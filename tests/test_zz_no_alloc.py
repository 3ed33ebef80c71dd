"""The forward-residual entry point that allocates nothing.

Some callers cannot allocate device memory: their device memory is owned by
another allocator's pool with a fixed budget, or they run in loops where
cudaMalloc's implicit device synchronisation is not allowed.  For them
at_forward_residual_noalloc takes its reduction scratch from a fixed array in
the library.  Here it is called through the C-ABI twice in a row (different
inputs each time, so the second call starts from the first call's leftovers in
the shared array) and compared with the existing forward projector, at_forward:
the residual must match it exactly (same kernel arithmetic), and the energy,
summed from the stored FP32 residual's exact squares, the FP64 sum of those
squares to 1e-12 relative.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(L, engine, arr):
    p = C.c_void_p()
    engine.engine._check("at_dev_alloc", L.at_dev_alloc(C.byref(p), arr.nbytes))
    engine.engine._check("h2d", L.at_memcpy_h2d(p, arr.ctypes.data, arr.nbytes, None))
    return p


def _host(L, engine, dptr, shape, dtype):
    out = np.zeros(shape, dtype)
    engine.engine._check("d2h", L.at_memcpy_d2h(out.ctypes.data, dptr, out.nbytes, None))
    engine.engine._check("sync", L.at_stream_sync(None))
    return out


def _plan(engine, kind):
    if kind == "fan":
        return engine.Plan.fan(engine.FanGeometry.covering(256, 1.0, 360, 512))
    if kind == "rays":  # a non-uniform view table, given ray by ray
        ang = np.sort(np.random.default_rng(5).uniform(0.0, 360.0, 150))
        return engine.Plan.rays(engine.RayGeometry.fan_from_view_table(128, 1.0, 200, ang, det_pitch_deg=0.19))
    if kind == "cone":
        return engine.Plan.cone(engine.ConeGeometry(32, 32, 24, 1.0, 40, 28, 36, 1.6, 80.0, 150.0))
    return engine.Plan.goldnc()


def _image(engine, plan, seed):
    if len(plan.img_shape) == 3:
        nz, n, _ = plan.img_shape
        return engine.phantom.csg_phantom(n, nz, seed=seed, n_parts=4, n_voids=3)
    return engine.phantom.ellipse_phantom(plan.img_shape[0], seed=seed, n_random=5)


@pytest.mark.parametrize("kind", ["fan", "rays", "cone", "goldnc"])
def test_noalloc_forward_residual_matches_forward(engine, kind):
    L = engine.lib()
    plan = _plan(engine, kind)
    shape = plan.sino_shape
    rng = np.random.default_rng(77)
    bufs = []
    for call in range(2):
        img = _image(engine, plan, 50 + call)
        g = (rng.random(shape) * 4.0).astype(np.float32)
        d_img, d_g = _dev(L, engine, img), _dev(L, engine, g)
        d_r, d_e = _dev(L, engine, np.zeros(shape, np.float32)), _dev(L, engine, np.zeros(1))
        bufs += [d_img, d_g, d_r, d_e]
        rc = L.at_forward_residual_noalloc(plan.handle, d_img, d_g, d_r, d_e, None)
        assert rc == 0, L.at_last_error().decode()
        r = _host(L, engine, d_r, shape, np.float32)
        energy = float(_host(L, engine, d_e, (1,), np.float64)[0])
        # the existing entry point
        d_s = _dev(L, engine, np.zeros(shape, np.float32))
        bufs.append(d_s)
        engine.engine._check("at_forward", L.at_forward(plan.handle, d_img, d_s, None))
        a = _host(L, engine, d_s, shape, np.float32)
        np.testing.assert_array_equal(r, g - a)
        ref = float(np.sum(r.astype(np.float64) ** 2))
        assert abs(energy - ref) <= 1e-12 * ref
    for p in bufs:
        L.at_dev_free(p)


def test_noalloc_rejects_plans_beyond_its_scratch(engine):
    L = engine.lib()
    plan = engine.Plan.fan(engine.FanGeometry.covering(16, 1.0, 4096, 4096))
    # real buffers of the plan's sizes, so that no call can ever reach a
    # kernel with an invalid address; the size check rejects the call first
    img = np.zeros(plan.img_shape, np.float32)
    sino = np.zeros(plan.sino_shape, np.float32)
    bufs = [_dev(L, engine, img), _dev(L, engine, sino), _dev(L, engine, sino), _dev(L, engine, np.zeros(1))]
    rc = L.at_forward_residual_noalloc(plan.handle, *bufs, None)
    assert rc == -1
    assert "scratch" in L.at_last_error().decode()
    np.testing.assert_array_equal(_host(L, engine, bufs[2], plan.sino_shape, np.float32), sino)
    for p in bufs:
        L.at_dev_free(p)
