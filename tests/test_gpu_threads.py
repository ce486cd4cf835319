"""Separate contexts on separate host threads: two renderers, each driven by
its own thread with its own scene, views and tuning, rebin concurrently (the
C calls release the interpreter lock) and give the same keys, values, tile
ranges and images as the same work done one context at a time."""
import threading

import numpy as np
import pytest

from gs3d import GaussianSplatRenderer, Scene, scenes

pytestmark = pytest.mark.gpu


def _job(seed, tile, w, h):
    data = scenes.scene_clusters(200_000, seed=seed, sh_degree=1)
    eyes = scenes.orbit_eyes(4, radius=10.0, jitter_deg=15.0, seed=seed)
    views = [(0, scenes.camera_at(e, w, h).getUniformData(w, h), w, h) for e in eyes]
    return data, views, tile


def _render(r, job, reps):
    data, views, tile = job
    out = []
    for _ in range(reps):
        r.setTuning(tile, 8, 0)
        r.rebinBatch(views)
        out = [(r.readViewImage(v).copy(), r.readViewRefs(v)) for v in range(len(views))]
    return out


def _same(a, b):
    for (ia, (ka, va, ca)), (ib, (kb, vb, cb)) in zip(a, b):
        assert np.array_equal(ia.view(np.uint16), ib.view(np.uint16))
        assert np.array_equal(ka, kb) and np.array_equal(va, vb) and np.array_equal(ca, cb)


def test_two_contexts_on_two_threads(built_lib):
    jobs = [_job(21, 16, 960, 540), _job(22, 32, 1280, 720)]
    rs = [GaussianSplatRenderer(Scene()) for _ in jobs]
    for r, job in zip(rs, jobs):
        r.init()
        r.setSplatData(job[0])
    try:
        want = [_render(r, job, 1) for r, job in zip(rs, jobs)]  # one at a time
        got, errors = [None, None], []

        def run(i):
            try:
                got[i] = _render(rs[i], jobs[i], 5)
            except Exception as e:  # reported below, on the main thread
                errors.append(e)

        ts = [threading.Thread(target=run, args=(i,)) for i in range(2)]
        for t in ts:
            t.start()
        for t in ts:
            t.join(300)
        assert not errors, errors
        for i in range(2):
            _same(got[i], want[i])
    finally:
        for r in rs:
            r.destroy()
