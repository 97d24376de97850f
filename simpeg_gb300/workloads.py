"""Seeded synthetic DC workloads (meshes, conductivity models, surveys).

These stand in for field data: the reference publishes no benchmark dataset
for this path.  Every builder takes a seed and uses ``np.random.default_rng``.

* ``block_model_survey``     -- 32x32x16 cells of 10 m, 0.01 S/m background with
  one 0.1 S/m and one 0.001 S/m block (6x6x4 cells each), dipole-dipole line
  along x: 20 sources x 15 receivers = 300 data.
* ``scale_forward``          -- 128x128x64 cells (~1.07 M), 5 m core cells, 8
  padding cells at x1.3 on each x/y side and at the bottom, log10 sigma a
  Gaussian random field (mean -2, std 0.5, correlation 10 cells), 256
  pole sources on a 16x16 surface grid, 40 dipole receivers each.
* ``differentiation``        -- 96x96x48 cells, m = ln sigma (ExpMap), 128
  dipole sources x 30 receivers.
"""

from __future__ import annotations

import numpy as np

from .mesh import TensorMesh
from .resistivity import receivers, sources
from .resistivity.survey import Survey


def gaussian_random_field(shape, corr_cells, rng):
    """FFT-filtered white noise with a Gaussian kernel (std corr_cells/2 cells), zero mean, unit std."""
    w = rng.standard_normal(shape)
    s = corr_cells / 2.0
    F = np.fft.fftn(w)
    filt = np.ones(shape)
    for ax, n in enumerate(shape):
        f = np.fft.fftfreq(n)
        g = np.exp(-2.0 * (np.pi * f * s) ** 2)
        sh = [1] * len(shape)
        sh[ax] = n
        filt = filt * g.reshape(sh)
    out = np.real(np.fft.ifftn(F * filt))
    out -= out.mean()
    out /= out.std()
    return out


def log10_sigma_field(mesh, rng, mean=-2.0, std=0.5, corr_cells=10.0):
    nx, ny, nz = mesh.shape_cells
    g = gaussian_random_field((nx, ny, nz), corr_cells, rng)
    return (mean + std * g).ravel(order="F")


def padded_mesh(ncore_xy, ncore_z, core_h, npad=8, factor=1.3):
    hxy = [(core_h, npad, -factor), (core_h, ncore_xy), (core_h, npad, factor)]
    hz = [(core_h, npad, -factor), (core_h, ncore_z)]
    return TensorMesh([hxy, hxy, hz], origin="CCN")


# ---------------------------------------------------------------- 32x32x16 block model
def block_model_survey(seed=0):
    rng = np.random.default_rng(seed)
    mesh = TensorMesh([[(10.0, 32)], [(10.0, 32)], [(10.0, 16)]], origin="CCN")
    nx, ny, nz = mesh.shape_cells
    sig = np.full((nx, ny, nz), 0.01)
    placed = []
    for val in (0.1, 0.001):
        for _ in range(1000):
            i0 = int(rng.integers(2, nx - 6 - 2 + 1))
            j0 = int(rng.integers(2, ny - 6 - 2 + 1))
            k0 = int(rng.integers(2, nz - 4 - 2 + 1))
            box = (i0, i0 + 6, j0, j0 + 6, k0, k0 + 4)
            if all(box[1] <= b[0] or b[1] <= box[0] or box[3] <= b[2] or b[3] <= box[2] or box[5] <= b[4]
                   or b[5] <= box[4] for b in placed):
                placed.append(box)
                sig[box[0]:box[1], box[2]:box[3], box[4]:box[5]] = val
                break
    sigma = sig.ravel(order="F")
    # stations every 10 m along x at y = 0, z = 0 (all on nodes); a = 20 m dipoles
    xs = -150.0 + 10.0 * np.arange(31)
    src_list = []
    for i in range(20):
        a, b = xs[i], xs[i + 2]
        cand = [j for j in range(i + 3, 29)] + [j for j in range(0, i - 2) if j + 2 <= i - 1]
        js = cand[:15]
        M = np.c_[xs[js], np.zeros(15), np.zeros(15)]
        N = np.c_[xs[np.array(js) + 2], np.zeros(15), np.zeros(15)]
        rx = receivers.Dipole(M, N)
        src_list.append(sources.Dipole([rx], np.r_[a, 0.0, 0.0], np.r_[b, 0.0, 0.0]))
    return mesh, sigma, Survey(src_list), placed


# ---------------------------------------------------------------- 1M-cell forward
def scale_forward(seed=1, n_side=16, n_rx=40, ncore_xy=112, ncore_z=56, core_h=5.0):
    rng = np.random.default_rng(seed)
    mesh = padded_mesh(ncore_xy, ncore_z, core_h)
    log10s = log10_sigma_field(mesh, rng)
    sigma = 10.0 ** log10s
    half = core_h * ncore_xy / 2.0
    # 16x16 pole grid over the core, snapped to nodes
    g = np.round(np.linspace(-0.8 * half, 0.8 * half, n_side) / core_h) * core_h
    src_list = []
    nst = n_rx + 1
    xr = np.round(np.linspace(-0.9 * half, 0.9 * half, nst) / core_h) * core_h
    for yv in g:
        for xv in g:
            M = np.c_[xr[:-1], np.full(n_rx, yv), np.zeros(n_rx)]
            N = np.c_[xr[1:], np.full(n_rx, yv), np.zeros(n_rx)]
            src_list.append(sources.Pole([receivers.Dipole(M, N)], np.r_[xv, yv, 0.0]))
    return mesh, sigma, Survey(src_list)


# ---------------------------------------------------------------- differentiation
def differentiation(seed=2, n_src=128, n_rx=30, ncore_xy=80, ncore_z=40, core_h=5.0):
    rng = np.random.default_rng(seed)
    mesh = padded_mesh(ncore_xy, ncore_z, core_h)
    m = np.log(10.0) * log10_sigma_field(mesh, rng)
    half = core_h * ncore_xy / 2.0
    n_lines = 8
    per_line = n_src // n_lines
    ys = np.round(np.linspace(-0.7 * half, 0.7 * half, n_lines) / core_h) * core_h
    xs = np.round(np.linspace(-0.8 * half, 0.8 * half, per_line + n_rx + 3) / core_h) * core_h
    src_list = []
    for yv in ys:
        for i in range(per_line):
            a, b = xs[i], xs[i + 1]
            js = np.arange(i + 2, i + 2 + n_rx)
            M = np.c_[xs[js], np.full(n_rx, yv), np.zeros(n_rx)]
            N = np.c_[xs[js + 1], np.full(n_rx, yv), np.zeros(n_rx)]
            src_list.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[a, yv, 0.0], np.r_[b, yv, 0.0]))
    return mesh, m, Survey(src_list)


# ---------------------------------------------------------------- Gauss-Newton step
def gauss_newton(seed=4, n_lines=16, src_per_line=32, n_rx=48, ncore_xy=144, ncore_z=72, core_h=5.0):
    """160x160x80 cells (~2.05 M), m = ln sigma, 512 dipole sources x 48 dipole receivers.

    16 survey lines along x, stations every 5 m; source i of a line is the dipole
    (station i, i+1) and its receivers are the dipoles (i+1+n, i+2+n), n = 1..48.
    Returns mesh, true model, starting model (the true field's mean) and survey.
    """
    rng = np.random.default_rng(seed)
    mesh = padded_mesh(ncore_xy, ncore_z, core_h)
    m_true = np.log(10.0) * log10_sigma_field(mesh, rng)
    m0 = np.full(mesh.n_cells, m_true.mean())
    half = core_h * ncore_xy / 2.0
    ys = np.round(np.linspace(-0.75 * half, 0.75 * half, n_lines) / core_h) * core_h
    nst = src_per_line + n_rx + 2
    x0 = -np.round((nst * core_h) / 2.0 / core_h) * core_h
    xs = x0 + core_h * np.arange(nst)
    src_list = []
    for yv in ys:
        for i in range(src_per_line):
            js = i + 1 + np.arange(1, n_rx + 1)
            M = np.c_[xs[js], np.full(n_rx, yv), np.zeros(n_rx)]
            N = np.c_[xs[js + 1], np.full(n_rx, yv), np.zeros(n_rx)]
            src_list.append(sources.Dipole([receivers.Dipole(M, N)], np.r_[xs[i], yv, 0.0],
                                           np.r_[xs[i + 1], yv, 0.0]))
    return mesh, m_true, m0, Survey(src_list)


# ---------------------------------------------------------------- batched uneven problems
def batched_problems(seed=5, n=64, lo=(32, 32, 16), hi=(96, 96, 64), h=10.0, src_range=(16, 128), n_rx=20):
    """n independent problems: cell counts log-uniform per axis between lo and hi (even),
    sources uniform in src_range (pole sources on a surface line), n_rx dipoles each,
    conductivity = random field (log10 mean -2, std 0.5, correlation 6 cells) + one 0.1 S/m block."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        dims = [int(2 * round(np.exp(rng.uniform(np.log(a), np.log(b))) / 2)) for a, b in zip(lo, hi)]
        mesh = TensorMesh([[(h, d)] for d in dims], origin="CCN")
        log10s = log10_sigma_field(mesh, rng, corr_cells=6.0).reshape(dims, order="F")
        bx, by, bz = [max(2, d // 5) for d in dims]
        i0, j0, k0 = [int(rng.integers(1, d - b - 1)) for d, b in zip(dims, (bx, by, bz))]
        log10s[i0:i0 + bx, j0:j0 + by, k0:k0 + bz] = -1.0
        sigma = 10.0 ** log10s.ravel(order="F")
        ns = int(rng.integers(src_range[0], src_range[1] + 1))
        half_x = h * dims[0] / 2.0
        half_y = h * dims[1] / 2.0
        xs = np.round(np.linspace(-0.8 * half_x, 0.8 * half_x, n_rx + 1) / h) * h
        src_list = []
        for s in range(ns):
            yv = np.round(rng.uniform(-0.7 * half_y, 0.7 * half_y) / h) * h
            xv = np.round(rng.uniform(-0.8 * half_x, 0.8 * half_x) / h) * h
            M = np.c_[xs[:-1], np.full(n_rx, yv), np.zeros(n_rx)]
            N = np.c_[xs[1:], np.full(n_rx, yv), np.zeros(n_rx)]
            src_list.append(sources.Pole([receivers.Dipole(M, N)], np.r_[xv, yv, 0.0]))
        out.append((mesh, sigma, Survey(src_list)))
    return out
