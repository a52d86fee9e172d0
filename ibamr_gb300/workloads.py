"""Seeded synthetic workloads with the shapes of the reference benchmark
configurations (immersed-boundary marker sets on periodic grids).

No dataset is involved: every workload is generated from a fixed seed.
"""

import numpy as np

SEED = 20261204


def ellipse_springs(n=256):
    """2D closed ellipse (semi-axes 0.25/0.20 about (0.5, 0.5)), equispaced
    angles, and linear-spring forces between neighbours (stiffness 1, rest
    length 0): F_k = (X_{k+1} - X_k) + (X_{k-1} - X_k)."""
    th = 2.0 * np.pi * np.arange(n) / n
    X = np.stack([0.5 + 0.25 * np.cos(th), 0.5 + 0.20 * np.sin(th)], axis=1)
    F = (np.roll(X, -1, axis=0) - X) + (np.roll(X, 1, axis=0) - X)
    return X.reshape(-1), F.reshape(-1)


def fibonacci_shell(n=200_000, N=128, radius=0.3, centre=0.5, seed=SEED + 2):
    """Sphere shell on a Fibonacci lattice with uniform jitter of 0.1 h."""
    rng = np.random.default_rng(seed)
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    phi = np.arange(n) * np.pi * (3.0 - np.sqrt(5.0))
    r = np.sqrt(1.0 - z * z)
    X = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1) * radius + centre
    h = 1.0 / N
    X += rng.uniform(-0.1 * h, 0.1 * h, size=X.shape)
    return X.reshape(-1)


def helices_and_uniform(n_fibres=64, per_fibre=25_000, n_uniform=400_000, seed=SEED + 3):
    """Clustered 3D marker set: helical fibres (radius 0.02, arc length 0.6,
    axial extent 0.15, i.e. about 4.6 turns, random orientation) packed into
    the sub-box [0.4, 0.6]^3, plus markers uniform in the unit cube."""
    rng = np.random.default_rng(seed)
    R, L, H = 0.02, 0.6, 0.15
    turns = np.sqrt(L * L - H * H) / (2.0 * np.pi * R)
    j = np.arange(per_fibre) / per_fibre
    pts = []
    for _ in range(n_fibres):
        a = rng.standard_normal(3)
        a /= np.linalg.norm(a)
        e1 = np.cross(a, [1.0, 0.0, 0.0] if abs(a[0]) < 0.9 else [0.0, 1.0, 0.0])
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(a, e1)
        half = 0.5 * H + R
        c = rng.uniform(0.4 + half, 0.6 - half, size=3)
        th = 2.0 * np.pi * turns * j
        zz = H * j - 0.5 * H
        P = c + R * np.cos(th)[:, None] * e1 + R * np.sin(th)[:, None] * e2 + zz[:, None] * a
        pts.append(P)
    pts.append(rng.uniform(0.0, 1.0, size=(n_uniform, 3)))
    X = np.concatenate(pts, axis=0)
    return np.ascontiguousarray(X.reshape(-1))


def fourier_curve(n, seed):
    """Closed curve r(t) = 0.25 + sum_{j=1..4} (a_j cos jt + b_j sin jt),
    a_j, b_j ~ N(0, 0.02), centred at (0.5, 0.5), equispaced t."""
    rng = np.random.default_rng(seed)
    a = rng.normal(0.0, 0.02, size=4)
    b = rng.normal(0.0, 0.02, size=4)
    t = 2.0 * np.pi * np.arange(n) / n
    r = 0.25 + sum(a[k] * np.cos((k + 1) * t) + b[k] * np.sin((k + 1) * t) for k in range(4))
    X = np.stack([0.5 + r * np.cos(t), 0.5 + r * np.sin(t)], axis=1)
    return X.reshape(-1)


def batched_2d(n_problems=512, seed=SEED + 4):
    """Independent 2D periodic problems: N uniform in {32,...,512}, marker
    counts log-uniform in [100, 20000] on random Fourier curves."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(n_problems):
        N = int(rng.choice([32, 64, 128, 256, 512]))
        n = int(np.floor(np.exp(rng.uniform(np.log(100.0), np.log(20000.0)))))
        out.append((N, fourier_curve(n, seed * 1000 + p)))
    return out


def serving_mix(n_sims=32, seed=SEED + 5):
    """Resident simulations of the serving workload: each 2D with N uniform in
    [64, 512] or 3D with N uniform in [32, 192] (equal odds), markers
    log-uniform in [1e3, 5e5] on a Fourier curve (2D) or a Fibonacci sphere
    shell (3D), forces and velocities N(0, 1).  Returns a list of (sid, dim,
    N, X, F, u) with X and F FP64 and u FP32 of shape (dim,) + N[::-1]."""
    rng = np.random.default_rng(seed)
    out = []
    for sid in range(n_sims):
        dim = 2 if rng.uniform() < 0.5 else 3
        N = int(rng.integers(64, 513)) if dim == 2 else int(rng.integers(32, 193))
        n = int(np.floor(np.exp(rng.uniform(np.log(1e3), np.log(5e5)))))
        if dim == 2:
            X = fourier_curve(n, 5000 + sid)
        else:
            X = fibonacci_shell(n, N, seed=6000 + sid)
        F = rng.standard_normal(n * dim)
        u = rng.standard_normal([dim] + [N] * dim).astype(np.float32)
        out.append((sid, dim, [N] * dim, X, F, u))
    return out


def touched_faces(X, dim, N, kernel_width, side=True):
    """|T|: distinct grid values inside the support of at least one marker
    (per component, summed), computed with torch on the markers' device."""
    import torch

    Xt = torch.as_tensor(X, device="cuda").view(-1, dim)
    total = 0
    comps = range(dim) if side else [None]
    for c in comps:
        base = []
        for d in range(dim):
            t = Xt[:, d] * N[d] + (0.5 if (side and d == c) else 0.0)
            if kernel_width % 2 == 0:
                b = torch.floor(t + 0.5).long() - kernel_width // 2
            else:
                b = torch.floor(t).long() - kernel_width // 2
            base.append(b)
        mark = torch.zeros(int(np.prod(N)), dtype=torch.bool, device="cuda")
        offs = torch.arange(kernel_width, device="cuda")
        for o in torch.cartesian_prod(*([offs] * dim)):
            lin = torch.zeros_like(base[0])
            for d in reversed(range(dim)):
                lin = lin * N[d] + torch.remainder(base[d] + o[d], N[d])
            mark[lin] = True
        total += int(mark.sum().item())
    return total
