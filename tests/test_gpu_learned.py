"""Learned raster schedule: the cost-MLP kernels against the float64
oracle, the schedule's image invariance, and what the trained network gains
over the key count it falls back to."""
import ctypes as C

import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, learned, scenes
from gs3d import _lib
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(t):
    return C.c_void_p(t.data_ptr())


def test_mlp_kernels_match_float64_oracle(built_lib):
    lib = _lib.load()
    rng = np.random.default_rng(11)
    p = learned.init_params(3, 0.7)
    p[1024:1088] = rng.normal(0, 0.1, 64)  # non-zero biases
    n = 300
    x = rng.normal(0, 1, (n, 16)).astype(np.float32)
    t = rng.normal(2, 1, n).astype(np.float32)
    dp, dx, dt = (torch.from_numpy(a).cuda() for a in (p, x, t))
    acts = torch.empty((n, 129), device="cuda")
    y = torch.empty(n, device="cuda")
    g = torch.zeros(len(p), device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.gs3d_mlp_forward(dev(dp), dev(dx), n, dev(acts), dev(y), s) == 0
    assert lib.gs3d_mlp_backward(dev(dp), dev(dx), dev(acts), dev(dt), n, dev(g), s) == 0
    yi = torch.empty(n, device="cuda")
    assert lib.gs3d_mlp_infer(dev(dp), dev(dx), n, dev(yi), s) == 0
    torch.cuda.synchronize()
    y_ref, _, _ = mlp_oracle.forward(p, x)
    g_ref = mlp_oracle.grad(p, x, t)
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=1e-4, atol=1e-4)
    gd = g.cpu().numpy()
    assert np.abs(gd - g_ref).max() <= 1e-3 * np.abs(g_ref).max() + 1e-6
    # bf16 tensor-core inference: within bf16 rounding of the f32 forward
    assert np.abs(yi.cpu().numpy() - y_ref).max() <= 0.05 * (np.abs(y_ref).max() + 1)


@pytest.fixture(scope="module")
def renderer(built_lib):
    r = GaussianSplatRenderer(Scene())
    r.init()
    yield r
    r.destroy()


def test_learned_schedule_keeps_image(renderer):
    r = renderer
    data = scenes.scene_clusters(200_000, seed=5, sh_degree=1)
    w, h = 1280, 720
    u = scenes.camera_at((2.0, 1.0, 10.0), w, h).getUniformData(w, h)
    r.setSplatData(data)
    r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
    r.rebin(data.splatCount, 80, 45, w, h, u)
    img0, c0 = r.readImage(), r.readBuffer("tile_costs")
    p = learned.init_params(1)
    assert r.lib.gs3d_set_cost_model(r.ctx, p.ctypes.data_as(C.c_void_p),
                                     np.zeros(16, np.float32).ctypes.data_as(C.c_void_p),
                                     np.ones(16, np.float32).ctypes.data_as(C.c_void_p)) == 0
    r.setSchedule(_lib.SCHEDULE_LEARNED)
    r.rebin(data.splatCount, 80, 45, w, h, u)
    img1, c1 = r.readImage(), r.readBuffer("tile_costs")
    r.setSchedule(_lib.SCHEDULE_ROW_MAJOR)
    assert np.array_equal(img0.view(np.uint16), img1.view(np.uint16))
    assert np.array_equal(c0, c1)


def test_trained_network_beats_key_count(renderer):
    """Trained on 240 random poses, evaluated on 60 held-out ones of a dense
    1M-splat scene: the network's log-cost error is below that of the best
    linear predictor from the key count alone (the quantity the fallback
    schedule orders by), and it ranks tiles better."""
    r = renderer
    data = scenes.scene_clusters(1_000_000, seed=6, sh_degree=0)
    r.setSplatData(data)
    w, h = 960, 544
    eyes = scenes.random_eyes(300, 8.0, 16.0, seed=6)
    us = [scenes.camera_at(e, w, h).getUniformData(w, h) for e in eyes]
    x, t, k = learned.collect(r.lib, r.ctx, us, w, h)
    xtr, ttr = x[:240].reshape(-1, 16), t[:240].reshape(-1)
    res = learned.train(r.lib, xtr, ttr, steps=3000, batch=65536, lr=5e-3)
    m = learned.evaluate(r.lib, res, x[240:], t[240:], k[240:])
    print("held-out:", m)
    assert res.losses[-1] < res.losses[0]
    assert m["mlp_mae_log"] < m["keycount_mae_log"]
    assert m["mlp_spearman"] > m["keycount_spearman"]
    assert learned.gate(m)
