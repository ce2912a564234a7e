"""The three seed initialisers of the reference (backend/main.py:68-326):
dichotomy (the default), sphere tracing and gradient descent, on a small
sphere-like network, with and without extra half-space constraints."""
import pytest
import torch

from analyticmesh_gb300 import get_boundary, seeds as S, workloads as wl

AVG_EPS = 1e-3  # the initialisers' default stopping tolerance on mean |f - iso|
METHODS = {"dichotomy": S.dichotomy, "sphere_tracing": S.sphere_tracing, "gradient_descent": S.gradient_descent}


@pytest.fixture(scope="module")
def model():
    return wl.geometric([32, 32], 7)


@pytest.mark.parametrize("method", list(METHODS))
def test_seed_points_lie_near_the_level_set(model, method):
    g = torch.Generator().manual_seed(0)
    p = METHODS[method](model, 0.0, init_num=256, generator=g)
    assert p.dim() == 2 and p.shape[1] == 3 and 0 < p.shape[0] <= 256
    if method != "sphere_tracing":  # sphere tracing keeps the points that stay inside the ball
        assert p.shape[0] == 256
    with torch.no_grad():
        f = model(p).reshape(-1)
    # the initialisers stop on the mean error of the batch they refine; a
    # subset of it may sit slightly above that
    assert f.abs().mean() < 2 * AVG_EPS
    assert ((p ** 2).sum(1) < 1.0 + 1e-6).all()


@pytest.mark.parametrize("method", list(METHODS))
def test_seed_points_respect_extra_constraints_and_iso(model, method):
    w, b = get_boundary("cube", min_vert=[-1, -1, 0.0], max_vert=[1, 1, 1])
    g = torch.Generator().manual_seed(0)
    p = METHODS[method](model, 0.05, init_num=128, w_extra_constraints=w, b_extra_constraints=b, generator=g)
    assert p.shape[0] > 0
    assert ((p @ w.t() + b) < 0).all()
    with torch.no_grad():
        f = model(p).reshape(-1) - 0.05
    assert f.abs().mean() < 2 * AVG_EPS


def test_dichotomy_is_reproducible_with_a_generator(model):
    a = S.dichotomy(model, 0.0, init_num=64, generator=torch.Generator().manual_seed(3))
    b = S.dichotomy(model, 0.0, init_num=64, generator=torch.Generator().manual_seed(3))
    assert torch.equal(a, b)


def test_gradient_descent_rejects_unknown_loss(model):
    with pytest.raises(ValueError):
        S.gradient_descent(model, 0.0, init_num=8, loss_type="huber")


def test_dichotomy_pinned_to_the_reference_draws():
    """The reference's own dichotomy (backend/main.py:252-326), run with its
    global RNGs seeded, gave tests/golden/seeds_dichotomy.npz
    (tests/golden/make_seed_golden.py); with the same draws -- a torch
    generator seeded like the global one, a random.Random seeded like
    Python's -- this implementation gives the same points, bit for bit."""
    import os
    import random

    import numpy as np

    from analyticmesh_gb300 import seeds, workloads as wl

    here = os.path.dirname(os.path.abspath(__file__))
    gold = np.load(os.path.join(here, "golden", "seeds_dichotomy.npz"))
    cases = [(7, [32, 32], 0.0, 256, 1024, 5), (12, [48, 48, 48], 0.05, 200, 2048, 9)]
    for c, (nseed, widths, iso, n, tries, seed) in enumerate(cases):
        model = wl.geometric(widths, nseed, perturb=0.05 if len(widths) > 2 else 0.0).float().eval()
        with torch.no_grad():
            pts = seeds.dichotomy(model, iso, init_num=n, try_pts_num=tries, init_ball_radius=1.0, iter_max=100,
                                  avg_eps=1e-3, time_out=60, generator=torch.Generator().manual_seed(seed),
                                  rng=random.Random(seed))
        assert np.array_equal(pts.numpy(), gold["points%d" % c]), c
