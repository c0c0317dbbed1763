"""The seeded request stream of the serving workload: the vectorised
generator gives exactly the requests of a draw-at-a-time generator over the
same counter-hash stream (same arrival times, scenes, sizes, cameras and
depth-of-field flags)."""
import math

import numpy as np

from swegl_gb300 import scenes as S


def _one_at_a_time(n, seed, rate=2000.0, n_scenes=8, radius=35.0, min_wh=(64, 64), max_wh=(3840, 2160),
                   dof_p=0.5):
    rng = S.Rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        u = rng.uniform(0.0, 1.0, 1)[0]
        t += -math.log(1.0 - u) / rate
        k = int(rng.integers(0, n_scenes - 1, 1)[0])
        w = S.log_uniform_int(rng, min_wh[0], max_wh[0])
        h = S.log_uniform_int(rng, min_wh[1], max_wh[1])
        m, c = S.camera_on_sphere(rng, radius)
        v = S.view_for(w, h, m, c)
        v.dof = bool(rng.uniform(0.0, 1.0, 1)[0] < dof_p)
        out.append((t, k, v))
    return out


def test_vectorised_stream_equals_draw_at_a_time():
    for seed in (60, 61, 70):
        a = _one_at_a_time(300, seed)
        b = S.serving_requests(300, seed=seed)
        assert len(a) == len(b)
        for (ta, ka, va), (tb, kb, vb) in zip(a, b):
            assert ta == tb and ka == kb
            assert (va.w, va.h, va.dof) == (vb.w, vb.h, vb.dof)
            assert np.array_equal(va.view, vb.view) and np.array_equal(va.proj, vb.proj)
            assert np.array_equal(va.camera_pos, vb.camera_pos)
