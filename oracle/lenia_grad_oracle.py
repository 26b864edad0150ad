"""Gradient oracle for the Lenia rollout -- TEST INFRASTRUCTURE ONLY.

leniax differentiates its rollout with jax.grad (runner.py:363-448); jax is
not installed here, so this restates the same graph -- FFT potential
(core.py:52-102), growth (growth_functions.py:6-82), one-kernel weighting
(core.py:202-242) and get_state (core.py:245-319, the v1 clip with its
straight-through gradient, core.py:267-270) -- in float64 torch on the CPU and
lets torch.autograd stand in for jax.grad.  A 'mask' clip variant (true
derivative of clip) is provided for checks against central finite
differences, which ``fd_grad`` computes in float64.

Only tests/ and bench.py's CPU legs may import this module.
"""
import numpy as np
import torch


def growth(u, m, s, slug):
    if slug == 'gaussian':
        return 2 * torch.exp(-((u - m) / s)**2 / 2) - 1
    if slug == 'poly_quad4':
        return 2 * torch.clamp(1 - (u - m)**2 / (9 * s**2), min=0)**4 - 1
    if slug == 'gaussian_target':
        return torch.exp(-((u - m) / s)**2 / 2)
    raise NotImplementedError(slug)


def rollout(cells0, k_real, m, s, w, dt, steps, slug='gaussian', clip='ste', mean=True, state_slug='v1'):
    """cells0 [..., H, W] float64; k_real [H, W] fftshifted world-sized kernel.
    Returns the state after `steps` steps."""
    Kh = torch.fft.rfft2(k_real)
    x = cells0
    for _ in range(steps):
        u = torch.fft.irfft2(torch.fft.rfft2(x) * Kh, s=x.shape[-2:])
        g = growth(u, m, s, slug)
        f = (w * g) / w if mean else w * g
        if state_slug == 'v2':
            x = x * (1 - dt) + dt * f
        elif state_slug == 'simple':
            x = x + dt * f
        else:
            n = x + dt * f
            c = torch.clamp(n, 0., 1.)
            x = (n - n.detach() + c.detach()) if clip == 'ste' else c
    return x


def loss_and_grads(cells0, k_real, m, s, w, dt, steps, target, **kw):
    """MSE loss of the final state against `target` and its gradients with
    respect to (cells0, k_real, m, s, w), all float64."""
    leaves = [torch.as_tensor(v, dtype=torch.float64).clone().requires_grad_(True)
              for v in (cells0, k_real, m, s, w)]
    final = rollout(*leaves, dt, steps, **kw)
    loss = ((final - torch.as_tensor(target, dtype=torch.float64))**2).mean()
    grads = torch.autograd.grad(loss, leaves)
    return float(loss), [g.numpy() for g in grads]


def fd_grad(fn, x0, idx, h=1e-6):
    """Central finite difference of scalar fn at x0 along the flat indices idx."""
    out = []
    x0 = np.array(x0, dtype=np.float64)
    for i in idx:
        xp = x0.copy().reshape(-1)
        xm = x0.copy().reshape(-1)
        xp[i] += h
        xm[i] -= h
        out.append((fn(xp.reshape(x0.shape)) - fn(xm.reshape(x0.shape))) / (2 * h))
    return np.array(out)


# ---------------------------------------------------------------------------
# Several channels and kernels, any number of world axes
def rollout_general(cells0, k_real, gf, w, dt, steps, cin, slugs, clip='ste', mean=True, state_slug='v1'):
    """The general graph of leniax's update (core.py:52-319): per kernel k the
    potential real(ifftn(fftn(state[c_in(k)]) * fftn(k_real[k]))) over every
    world axis, growth per kernel, the [C, K] weighting (weighted_mean divides
    by the per-channel weight sums, weighted_sum does not; core.py:202-242),
    then get_state.  cells0 [..., C, *world]; k_real [K, *world]; gf [K, 2];
    w [C, K]; cin / slugs: the input channel and growth slug of each kernel.
    Returns the state after `steps` steps."""
    nd = k_real.dim() - 1
    world = tuple(k_real.shape[1:])
    axes = tuple(range(-nd, 0))
    Kh = torch.fft.rfftn(k_real, dim=axes)  # [K, *half]
    idx = torch.as_tensor(cin, dtype=torch.long)
    x = cells0
    for _ in range(steps):
        X = torch.fft.rfftn(x, dim=axes)  # [..., C, *half]
        U = torch.fft.irfftn(X.index_select(-(nd + 1), idx) * Kh, s=world, dim=axes)  # [..., K, *world]
        G = torch.stack([growth(U.select(-(nd + 1), k), gf[k, 0], gf[k, 1], slugs[k]) for k in range(len(cin))],
                        dim=-(nd + 1))
        Gm = G.movedim(-(nd + 1), -1)  # [..., *world, K]
        f = (Gm.unsqueeze(-2) * w).sum(-1)  # [..., *world, C]
        if mean:
            f = f / w.sum(-1)
        f = f.movedim(-1, -(nd + 1))  # [..., C, *world]
        if state_slug == 'v2':
            x = x * (1 - dt) + dt * f
        elif state_slug == 'simple':
            x = x + dt * f
        else:
            n = x + dt * f
            c = torch.clamp(n, 0., 1.)
            x = (n - n.detach() + c.detach()) if clip == 'ste' else c
    return x


def loss_and_grads_general(cells0, k_real, gf, w, dt, steps, target, cin, slugs, **kw):
    """MSE loss of the final state against `target` and its gradients with
    respect to (cells0, k_real, gf, w), in the dtype of the inputs."""
    leaves = [torch.as_tensor(v).clone().requires_grad_(True) for v in (cells0, k_real, gf, w)]
    final = rollout_general(*leaves, dt, steps, cin, slugs, **kw)
    loss = ((final - torch.as_tensor(target))**2).mean()
    grads = torch.autograd.grad(loss, leaves)
    return float(loss.detach()), [g.numpy() for g in grads]
