"""Analytic fields of the benchmark workloads (seeded, synthetic).

Formulas restated from src/utils/fields.h (rotation :142-151, Gaussian
:275-293) and src/applications/include/field_wrappers.h (rotated Gaussian
:31-56); the Taylor-Green variant and the random divergence-free Fourier
fields are the ones the benchmark configurations specify.
"""
import math

import numpy as np


def rotation(omega=2 * math.pi):
    """Solid-body rotation about the z axis through (0.5, 0.5, 0.5)."""
    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        return np.stack([omega * (0.5 - p[:, 1]), omega * (p[:, 0] - 0.5),
                         np.zeros(len(p))], axis=1)
    return fn


def gaussian(centre, sigma, amp=1.0):
    c = np.asarray(centre, dtype=np.float64)

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        r2 = ((p - c) ** 2).sum(axis=1)
        return (amp * np.exp(-r2 / (2.0 * sigma * sigma)))[:, None]
    return fn


def rotated_gaussian(centre, sigma, omega, t):
    """The Gaussian carried by the rotation for time t (exact solution)."""
    cx, cy, cz = centre
    th = omega * t
    x = 0.5 + (cx - 0.5) * math.cos(th) - (cy - 0.5) * math.sin(th)
    y = 0.5 + (cx - 0.5) * math.sin(th) + (cy - 0.5) * math.cos(th)
    return gaussian((x, y, cz), sigma)


def taylor_green():
    """u = (sin 2pi x cos 2pi y cos 2pi z, -cos 2pi x sin 2pi y cos 2pi z, 0)."""
    tp = 2 * math.pi

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        return np.stack([np.sin(tp * x) * np.cos(tp * y) * np.cos(tp * z),
                         -np.cos(tp * x) * np.sin(tp * y) * np.cos(tp * z),
                         np.zeros(len(p))], axis=1)
    return fn


def gaussian_blobs(rng, n, sigma_range=(0.03, 0.08), centre_range=(0.2, 0.8)):
    """Sum of n Gaussians with seeded centres and widths."""
    centres = rng.uniform(centre_range[0], centre_range[1], size=(n, 3))
    sigmas = rng.uniform(sigma_range[0], sigma_range[1], size=n)

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        out = np.zeros(len(p))
        for c, s in zip(centres, sigmas):
            out += np.exp(-((p - c) ** 2).sum(axis=1) / (2.0 * s * s))
        return out[:, None]
    fn.centres, fn.sigmas = centres, sigmas
    return fn


def fourier_modes(rng, kmax=4):
    """Divergence-free random Fourier modes on the periodic unit cube.

    Integer wave vectors 0 < |k| <= kmax (one of each +-k pair); cosine and
    sine amplitude vectors drawn N(0,1)/|k|^2 per component and projected
    orthogonal to k, so div v = 0 exactly.
    """
    ks = []
    r = int(kmax)
    for a in range(-r, r + 1):
        for b in range(-r, r + 1):
            for c in range(-r, r + 1):
                k = (a, b, c)
                n2 = a * a + b * b + c * c
                if 0 < n2 <= kmax * kmax and k > (0, 0, 0) and tuple(-x for x in k) < k:
                    ks.append(k)
    ks = np.array(ks, dtype=np.float64)
    kn = np.sqrt((ks ** 2).sum(axis=1))
    A = rng.standard_normal((len(ks), 3)) / (kn ** 2)[:, None]
    B = rng.standard_normal((len(ks), 3)) / (kn ** 2)[:, None]
    khat = ks / kn[:, None]
    A -= (A * khat).sum(axis=1)[:, None] * khat
    B -= (B * khat).sum(axis=1)[:, None] * khat
    return ks, A, B


def fourier_velocity(rng, kmax=4):
    """v(x) = sum_k A_k cos(2pi k.x) + B_k sin(2pi k.x) as a point function."""
    ks, A, B = fourier_modes(rng, kmax)
    return fourier_velocity_from_modes(ks, A, B, kmax)


def fourier_velocity_from_modes(ks, A, B, kmax=4):
    """Evaluated as Re sum_k (A_k - i B_k) e_x[k_x] e_y[k_y] e_z[k_z] with the
    per-axis exponentials tabulated once per call."""
    ki = ks.astype(int)
    r = int(kmax)
    coef = A - 1j * B

    def fn(p):
        p = np.asarray(p, dtype=np.float64).reshape(-1, 3)
        kk = np.arange(-r, r + 1)
        E = [np.exp(2j * math.pi * np.outer(p[:, a], kk)) for a in range(3)]  # [n, 2r+1]
        out = np.zeros((len(p), 3))
        # group modes by (k_y, k_z): sum over k_x first
        groups = {}
        for m, (kx, ky, kz) in enumerate(ki):
            groups.setdefault((ky, kz), []).append(m)
        for (ky, kz), ms in groups.items():
            eyz = E[1][:, ky + r] * E[2][:, kz + r]
            acc = np.zeros((len(p), 3), dtype=np.complex128)
            for m in ms:
                acc += E[0][:, ki[m, 0] + r, None] * coef[m][None, :]
            out += (acc * eyz[:, None]).real
        return out
    fn.modes = (ks, A, B)
    return fn


def fourier_velocity_grid(rng, n, kmax=4):
    """The same field sampled on the periodic grid i/n, SoA [3, n, n, n] (z, y, x)."""
    ks, A, B = fourier_modes(rng, kmax)
    spec = np.zeros((3, n, n, n // 2 + 1), dtype=np.complex128)
    # v = sum Re((A - iB) e^{2 pi i k.x}); irfftn of index (kz, ky, kx) -> array [z, y, x]
    for k, a, b in zip(ks.astype(int), A, B):
        kx, ky, kz = k
        coef = (a - 1j * b)
        if kx < 0 or (kx == 0 and (ky < 0 or (ky == 0 and kz < 0))):
            kx, ky, kz, coef = -kx, -ky, -kz, np.conj(coef)
        scale = 1.0 if kx > 0 else 1.0
        if kx == 0:
            # half-plane kx = 0: irfftn keeps both (ky,kz) and (-ky,-kz) slots
            spec[:, kz % n, ky % n, 0] += 0.5 * coef * n ** 3
            spec[:, (-kz) % n, (-ky) % n, 0] += 0.5 * np.conj(coef) * n ** 3
        else:
            spec[:, kz % n, ky % n, kx] += 0.5 * coef * n ** 3 * scale
    out = np.fft.irfftn(spec, s=(n, n, n), axes=(1, 2, 3))
    return np.ascontiguousarray(out)


def periodic_blob_grid(n, centre=(0.5, 0.5, 0.5), sigma=0.1):
    """Gaussian concentration on the periodic grid i/n, [n, n, n] (z, y, x)."""
    x = np.arange(n) / n
    g = [np.exp(-(x - c) ** 2 / (2 * sigma * sigma)) for c in centre]
    return np.ascontiguousarray(g[2][:, None, None] * g[1][None, :, None] * g[0][None, None, :])


def wall_tangent_perturbation(rng, nmodes=4):
    """Random smooth velocity perturbation whose x-component vanishes on the
    planes x = 0, 1/2, 1 (likewise y, z): it keeps every plane on which a
    Taylor-Green-type flow is tangent, so the perturbed flow moves no node
    across those planes (the SL step is smooth along such directions)."""
    amp = rng.standard_normal((3, nmodes))
    kk = rng.integers(1, 4, size=(3, nmodes, 2))
    ph = rng.uniform(0, 2 * math.pi, size=(3, nmodes, 2))

    def fn(p):
        p = np.asarray(p).reshape(-1, 3)
        out = np.zeros((len(p), 3))
        for a in range(3):
            o1, o2 = [b for b in range(3) if b != a]
            g = np.zeros(len(p))
            for m in range(nmodes):
                g += amp[a, m] * np.cos(2 * math.pi * kk[a, m, 0] * p[:, o1] + ph[a, m, 0]) * \
                    np.cos(2 * math.pi * kk[a, m, 1] * p[:, o2] + ph[a, m, 1])
            out[:, a] = np.sin(2 * math.pi * p[:, a]) * g
        return out
    return fn
