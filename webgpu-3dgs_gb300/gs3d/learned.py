"""Cost model of the learned raster schedule: data collection, training with
the library's hand-written MLP kernels, held-out evaluation and the fallback
gate.

The model (16 features -> 64 -> 64 -> 1, ReLU) predicts log(1 + cost) of a
tile, the cost being the splats the raster CTA iterates before the tile's
last pixel terminates, as the plain rasterizer records it in tile_costs.
Training runs entirely on the GPU: gs3d_mlp_forward / gs3d_mlp_backward /
gs3d_mlp_adam on device buffers (torch tensors serve only as allocations).
The schedule orders the persistent raster CTAs' work and never changes an
image; when the measured held-out error is above the model's bound, or the
model ranks tiles no better than the key count, the key-count schedule is
used instead.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .camera import camera_struct

P = _lib.MLP_PARAMS
F = _lib.MLP_FEATURES
H = _lib.MLP_HIDDEN


def init_params(seed: int = 0, bias_out: float = 0.0) -> np.ndarray:
    """He-initialised parameters in the library's layout."""
    rng = np.random.default_rng(seed)
    w1 = rng.normal(0.0, np.sqrt(2.0 / F), (H, F))
    w2 = rng.normal(0.0, np.sqrt(2.0 / H), (H, H))
    w3 = rng.normal(0.0, np.sqrt(1.0 / H), H)
    p = np.concatenate([w1.ravel(), np.zeros(H), w2.ravel(), np.zeros(H), w3, [bias_out]])
    return p.astype(np.float32)


def _dev(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _check(lib, rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed ({rc}): {lib.gs3d_last_error(None).decode()}")


def collect(lib, ctx, uniforms, width: int, height: int):
    """Renders every camera (72-float uniform) with the fused single-view
    rebin and returns device tensors (features [V, T, 16], log-costs [V, T],
    key counts [V, T])."""
    import torch
    feats, targets, counts = [], [], []
    for u in uniforms:
        cs = camera_struct(u)
        for _ in range(3):
            _check(lib, lib.gs3d_rebin(ctx, C.byref(cs), width, height), "rebin")
            rc = lib.gs3d_synchronize(ctx)
            if rc != _lib.ERR_CAPACITY:
                break
        if rc != 0:
            raise RuntimeError(lib.gs3d_last_error(ctx).decode())
        info = _lib.ViewInfo_t()
        lib.gs3d_get_view_info(ctx, 0, C.byref(info))
        T = info.tiles_x * info.tiles_y
        x = torch.empty((T, F), dtype=torch.float32, device="cuda")
        t = torch.empty(T, dtype=torch.float32, device="cuda")
        rc = lib.gs3d_tile_features(ctx, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()), T, 1)
        if rc != 0:
            raise RuntimeError(lib.gs3d_last_error(ctx).decode())
        _check(lib, lib.gs3d_synchronize(ctx), "features")
        feats.append(x)
        targets.append(t)
        counts.append(torch.expm1(x[:, 1]))  # feature 1 = log(1 + key count)
    return torch.stack(feats), torch.stack(targets), torch.stack(counts)


@dataclass
class TrainResult:
    params: np.ndarray
    mean: np.ndarray
    std: np.ndarray
    losses: list


def train(lib, x, t, steps: int = 3000, batch: int = 65536, lr: float = 5e-3,
          seed: int = 0) -> TrainResult:
    """Adam on mean squared error of log-cost, all arithmetic in the
    library's kernels.  x: [N, 16] raw features, t: [N] targets (device)."""
    import torch
    mean = x.mean(0)
    std = x.std(0)
    std = torch.where(std > 1e-6, std, torch.ones_like(std))
    xn = ((x - mean) / std).contiguous()
    params = torch.from_numpy(init_params(seed, float(t.mean()))).cuda()
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    g = torch.zeros_like(params)
    n = xn.shape[0]
    b = min(batch, n)
    acts = torch.empty((b, 2 * H + 1), dtype=torch.float32, device="cuda")
    y = torch.empty(b, dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(seed)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    losses = []
    for step in range(1, steps + 1):
        idx = torch.randint(0, n, (b,), device="cuda", generator=gen)
        xb = xn[idx].contiguous()
        tb = t[idx].contiguous()
        _check(lib, lib.gs3d_mlp_forward(_dev(params), _dev(xb), b, _dev(acts), _dev(y), stream),
               "mlp forward")
        g.zero_()
        _check(lib, lib.gs3d_mlp_backward(_dev(params), _dev(xb), _dev(acts), _dev(tb), b,
                                          _dev(g), stream), "mlp backward")
        cur_lr = lr * (0.1 ** (step / steps))  # exponential decay to lr / 10
        _check(lib, lib.gs3d_mlp_adam(_dev(params), _dev(m), _dev(v), _dev(g), P, cur_lr, 0.9,
                                      0.999, 1e-8, step, stream), "adam")
        if step % 100 == 0 or step == steps:
            losses.append(float(((y - tb) ** 2).mean()))
    return TrainResult(params.cpu().numpy(), mean.cpu().numpy(), std.cpu().numpy(), losses)


def predict(lib, params: np.ndarray, mean, std, x):
    """bf16 tensor-core inference (gs3d_mlp_infer) on raw features x [N, 16]."""
    import torch
    xn = ((x - torch.as_tensor(mean, device="cuda")) /
          torch.as_tensor(std, device="cuda")).contiguous()
    p = torch.from_numpy(np.ascontiguousarray(params, np.float32)).cuda()
    y = torch.empty(xn.shape[0], dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(lib, lib.gs3d_mlp_infer(_dev(p), _dev(xn), xn.shape[0], _dev(y), stream), "mlp infer")
    torch.cuda.synchronize()
    return y


def spearman(a: np.ndarray, b: np.ndarray) -> float:
    ra = np.argsort(np.argsort(a, kind="stable"), kind="stable").astype(np.float64)
    rb = np.argsort(np.argsort(b, kind="stable"), kind="stable").astype(np.float64)
    ra -= ra.mean()
    rb -= rb.mean()
    den = np.sqrt((ra * ra).sum() * (rb * rb).sum())
    return float((ra * rb).sum() / den) if den > 0 else 0.0


def evaluate(lib, res: TrainResult, x, t, counts) -> dict:
    """Held-out metrics of the model and of the key-count proxy (a linear fit
    of log-cost on log key count, fitted on the held-out set itself, i.e. the
    best the key count alone can do)."""
    V, T, _ = x.shape
    pred = predict(lib, res.params, res.mean, res.std, x.reshape(V * T, F)).reshape(V, T)
    pred, tt = pred.cpu().numpy(), t.cpu().numpy()
    lk = np.log1p(counts.cpu().numpy())
    A = np.stack([lk.ravel(), np.ones(lk.size)], 1)
    coef, *_ = np.linalg.lstsq(A, tt.ravel(), rcond=None)
    lin = (A @ coef).reshape(V, T)
    return {
        "mlp_mae_log": float(np.abs(pred - tt).mean()),
        "keycount_mae_log": float(np.abs(lin - tt).mean()),
        "mlp_spearman": float(np.mean([spearman(pred[i], tt[i]) for i in range(V)])),
        "keycount_spearman": float(np.mean([spearman(lk[i], tt[i]) for i in range(V)])),
    }


# A model whose held-out mean |log error| exceeds this is not used.
ERROR_BOUND = 0.5


def gate(metrics: dict, bound: float = ERROR_BOUND) -> bool:
    """True when the learned schedule may replace the key-count schedule."""
    return (metrics["mlp_mae_log"] <= bound and
            metrics["mlp_spearman"] >= metrics["keycount_spearman"])


def save(path, res: TrainResult, metrics: dict, bound: float = ERROR_BOUND, **extra) -> None:
    np.savez(path, params=res.params, mean=res.mean, std=res.std, bound=np.float32(bound),
             metrics=np.array([metrics[k] for k in sorted(metrics)], np.float64),
             metric_names=np.array(sorted(metrics)), **extra)


def load(path) -> tuple[np.ndarray, np.ndarray, np.ndarray, dict, float]:
    d = np.load(path)
    metrics = dict(zip([str(k) for k in d["metric_names"]], d["metrics"].tolist()))
    return d["params"], d["mean"], d["std"], metrics, float(d["bound"])


def checkpoint_for(tile_w: int, tile_h: int):
    """Committed cost model of the 3M-splat 1080p workload for a tile size,
    or None (the model's features and costs are per tile, so a model only
    applies to the tile size it was trained on)."""
    from pathlib import Path
    here = Path(__file__).resolve().parent
    name = {(16, 16): "cost_mlp_c1.npz", (32, 32): "cost_mlp_c1_t32.npz",
            (64, 32): "cost_mlp_c1_t64x32.npz",
            (32, 64): "cost_mlp_c1_t32x64.npz"}.get((tile_w, tile_h))
    return here / name if name and (here / name).exists() else None


def main(argv=None) -> None:
    """Trains the cost model of the headline workload (3M-splat cluster
    scene, 1920x1080, 16x16 tiles by default) on random poses at radius
    8-16 and writes the checkpoint:
    python -m gs3d.learned OUT.npz [--poses 10000] [--heldout 1000] [--tile 16 | WxH]"""
    import argparse
    import time

    import torch

    from .renderer import GaussianSplatRenderer, Scene
    from . import scenes

    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--poses", type=int, default=10000)
    ap.add_argument("--heldout", type=int, default=1000)
    ap.add_argument("--splats", type=int, default=3_000_000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--chunk", type=int, default=1000)
    ap.add_argument("--tile", default="16", help="square size or WxH")
    a = ap.parse_args(argv)
    r = GaussianSplatRenderer(Scene())
    r.init()
    tw, th = (int(v) for v in a.tile.split("x")) if "x" in a.tile else (int(a.tile),) * 2
    r.setTuning((tw, th), 8, 0)
    # colour does not change a tile's raster cost: SH degree 0 suffices
    r.setSplatData(scenes.scene_clusters(a.splats, seed=0, sh_degree=0))
    total = a.poses + a.heldout
    eyes = scenes.random_eyes(total, 8.0, 16.0, seed=12345)
    t0 = time.time()
    xs, ts, ks = [], [], []
    for c0 in range(0, total, a.chunk):
        us = [scenes.camera_at(e, a.width, a.height).getUniformData(a.width, a.height)
              for e in eyes[c0:c0 + a.chunk]]
        x, t, k = collect(r.lib, r.ctx, us, a.width, a.height)
        xs.append(x)
        ts.append(t)
        ks.append(k)
    x, t, k = torch.cat(xs), torch.cat(ts), torch.cat(ks)
    t_collect = time.time() - t0
    t0 = time.time()
    res = train(r.lib, x[:a.poses].reshape(-1, F), t[:a.poses].reshape(-1), steps=a.steps)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    m = evaluate(r.lib, res, x[a.poses:], t[a.poses:], k[a.poses:])
    ok = gate(m)
    print(f"collect {t_collect:.1f}s train {t_train:.1f}s held-out {m} gate {'pass' if ok else 'FAIL'}")
    save(a.out, res, m, poses=np.int64(a.poses), heldout=np.int64(a.heldout),
         workload=np.array(f"{a.splats} splats {a.width}x{a.height} tiles {tw}x{th}"),
         tile=np.array([tw, th], np.int64))
    r.destroy()


if __name__ == "__main__":
    main()
