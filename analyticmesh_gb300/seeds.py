"""Seed points on the zero level set, one per starting region.

Same procedures as the reference's initialisers (backend/main.py:68-326):
``dichotomy`` (default), ``sphere_tracing`` and ``gradient_descent``.  Every
random draw takes an explicit ``torch.Generator`` so runs are reproducible;
the reference draws from the global RNG and Python's ``random``.
"""
from __future__ import annotations

import time

import numpy as np
import torch


def constraints_filter(x, w_extra, b_extra, requires_index=False):
    """Keep points inside every extra half-space w.x + b < 0 (backend/main.py:68-80)."""
    if w_extra is not None and b_extra is not None and w_extra.shape[0] > 0 and x.shape[0] > 0:
        w = w_extra.to(dtype=x.dtype, device=x.device)
        b = b_extra.to(dtype=x.dtype, device=x.device)
        index = ((x @ w.t() + b.reshape(1, -1)) < 0).all(dim=1)
        return (x[index], index) if requires_index else x[index]
    return (x, torch.ones(x.shape[0], dtype=torch.bool, device=x.device)) if requires_index else x


def init_within_ball(init_num, init_ball_radius, w_extra=None, b_extra=None, generator=None, device="cpu"):
    """Uniform points in a ball by rejection (backend/main.py:83-91)."""
    pts = torch.zeros([0, 3], dtype=torch.float32)
    while pts.shape[0] < init_num:
        p = (torch.rand([init_num - pts.shape[0], 3], dtype=torch.float32, generator=generator) * 2 - 1) * init_ball_radius
        p = p[(p ** 2).sum(dim=1) < init_ball_radius ** 2]
        p = constraints_filter(p, w_extra, b_extra)
        pts = torch.cat([pts, p], dim=0)
    return pts.to(device)


class _Corr:
    """Correlation of the recent error history with time (backend/main.py:94-107)."""

    def __init__(self, hist_len):
        self.hist_len = hist_len
        self.arange = np.arange(hist_len)
        self.arr = []

    def push(self, value):
        if not self.arr:
            self.arr = [value] * self.hist_len
            return 1.0
        self.arr = [value] + self.arr[:-1]
        return np.corrcoef(np.array(self.arr), self.arange)[0, 1]


def dichotomy(model, iso, init_num=1024, w_extra_constraints=None, b_extra_constraints=None, try_pts_num=4096,
              init_ball_radius=1.0, iter_max=100, avg_eps=1e-3, time_out=60, provided_surfpts=None,
              provided_surfstd=None, generator=None, device="cpu", verbose=False, rng=None):
    """Pairs of opposite-sign samples, bisected until the mean |f - iso| is
    below ``avg_eps`` (backend/main.py:252-326).  Returns (init_num, 3) fp32.

    ``rng`` (a ``random.Random``): draw the pairs as the reference does, by
    ``rng.sample`` over the n_pos x n_neg products and a float division for
    the negative index -- with ``generator`` seeded like the reference's
    global torch RNG, the same points from the same draws."""
    t0 = time.time()
    neg = torch.zeros([0, 3], device=device)
    pos = torch.zeros([0, 3], device=device)
    while neg.shape[0] < init_num:
        if time.time() - t0 > time_out:
            raise RuntimeError("dichotomy cannot find solution within %s seconds" % time_out)
        if provided_surfpts is not None and provided_surfstd is not None:
            noise = torch.randn(provided_surfpts.shape, generator=generator, dtype=provided_surfpts.dtype)
            pts = (provided_surfpts + provided_surfstd * noise).to(device)
        else:
            pts = init_within_ball(try_pts_num, init_ball_radius, w_extra_constraints, b_extra_constraints,
                                   generator=generator, device=device)
        with torch.no_grad():
            val = model(pts).reshape(-1) - iso
        id_pos = torch.where(val > 0)[0]
        id_neg = torch.where(val < 0)[0]
        n_pos, n_neg = len(id_pos), len(id_neg)
        if n_pos and n_neg:
            n_range = n_pos * n_neg
            n_sample = min(init_num - neg.shape[0], n_range)
            if rng is not None:
                index = torch.tensor(rng.sample(range(n_range), n_sample))
                index_neg = (index / n_pos).long().to(device)
                index = index.to(device)
            else:
                index = torch.randperm(n_range, generator=generator)[:n_sample].to(device)
                index_neg = index // n_pos
            pos = torch.cat([pos, pts[id_pos[index % n_pos]]], dim=0)
            neg = torch.cat([neg, pts[id_neg[index_neg]]], dim=0)
            if verbose:
                print("(am) (dichotomy) n_pos = %d | n_neg = %d" % (n_pos, n_neg))
    mid = (neg + pos) / 2
    with torch.no_grad():
        for _ in range(iter_max):
            v = model(mid).reshape(-1) - iso
            if torch.abs(v).mean() < avg_eps:
                break
            lt = v < 0
            neg[lt] = mid[lt]
            pos[~lt] = mid[~lt]
            mid = (neg + pos) / 2
    return mid


def sphere_tracing(model, iso, init_num=1024, step_size_max=1.0, step_size_mul=0.5, step_size_min=1e-3,
                   w_extra_constraints=None, b_extra_constraints=None, init_ball_radius=1.0, avg_eps=1e-3,
                   hist_len=100, corr_min=0.1, time_out=60, generator=None, device="cpu", verbose=False):
    """Gradient steps p -= step * f * grad f (backend/main.py:113-178)."""
    step = step_size_max
    t0 = time.time()
    corr = _Corr(hist_len)
    while True:
        pts = init_within_ball(init_num, init_ball_radius, w_extra_constraints, b_extra_constraints,
                               generator=generator, device=device)
        old = 1e10
        done = False
        while True:
            pts = pts.detach().requires_grad_(True)
            pred = model(pts) - iso
            err = torch.abs(pred).mean()
            c = corr.push(err.item())
            if time.time() - t0 > time_out:
                raise RuntimeError("sphere_tracing cannot find solution within time=%s" % time_out)
            if err > old * 2 or not torch.isfinite(err) or err > 100 or c < corr_min or not np.isfinite(c):
                step *= step_size_mul
                if step < step_size_min:
                    raise RuntimeError("sphere_tracing cannot find solution")
                break
            old = err
            if err < avg_eps:
                done = True
                break
            grad = torch.autograd.grad(pred, pts, grad_outputs=torch.ones_like(pred))[0]
            with torch.no_grad():
                pts = pts - step * pred * grad
        if done:
            break
    pts = pts.detach()
    pts = pts[(pts ** 2).sum(dim=1) < init_ball_radius ** 2]
    return constraints_filter(pts, w_extra_constraints, b_extra_constraints)


def gradient_descent(model, iso, init_num=1024, lr_max=1e-2, lr_mul=0.3, lr_min=1e-5, corr_min=0.1, hist_len=100,
                     loss_type="l1", optimizer_type="adam", accept_bad=True, w_extra_constraints=None,
                     b_extra_constraints=None, init_ball_radius=1.0, batch_mul=2, avg_eps=1e-3, time_out=60,
                     generator=None, device="cpu", verbose=False):
    """Minimise |f - iso| over the points with Adam/SGD (backend/main.py:181-249)."""
    if loss_type == "smooth_l1":
        a = avg_eps * 10
        loss_fn = lambda x: (torch.where(torch.abs(x / a) < 1, 0.5 * (x / a) ** 2, torch.abs(x / a) - 0.5) * a).mean()
    elif loss_type == "l1":
        loss_fn = lambda x: torch.abs(x).mean()
    elif loss_type == "l2":
        loss_fn = lambda x: (x ** 2).mean()
    else:
        raise ValueError("no such loss_type: %s" % loss_type)
    t0 = time.time()
    out = torch.zeros([0, 3], device=device)
    while out.shape[0] < init_num:
        p = init_within_ball(int((init_num - out.shape[0]) * batch_mul), init_ball_radius, w_extra_constraints,
                             b_extra_constraints, generator=generator, device=device).requires_grad_()
        opt = torch.optim.Adam([p], lr=lr_max) if optimizer_type == "adam" else torch.optim.SGD([p], lr=lr_max, momentum=0.9)
        err = 1e9
        corr = _Corr(hist_len)
        first = True
        pred = None
        while err > avg_eps:
            if not first:
                loss = loss_fn(pred)
                opt.zero_grad()
                loss.backward()
                opt.step()
            pred = model(p) - iso
            err = torch.abs(pred).mean().item()
            c = corr.push(err)
            first = False
            if time.time() - t0 > time_out:
                raise RuntimeError("gradient_descent cannot find solution within %s seconds" % time_out)
            if c < corr_min:
                corr = _Corr(hist_len)
                for g in opt.param_groups:
                    g["lr"] *= lr_mul
                if opt.param_groups[0]["lr"] < lr_min:
                    break
        if opt.param_groups[0]["lr"] >= lr_min or accept_bad:
            q = constraints_filter(p.detach(), w_extra_constraints, b_extra_constraints)
            out = torch.cat([out, q[: init_num - out.shape[0]]], dim=0)
    return out
