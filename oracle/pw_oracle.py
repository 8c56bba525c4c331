"""TEST INFRASTRUCTURE -- numpy restatement of CP2K's multigrid transfer
between the realspace level grids and the plane-wave grid, the checker of
grid_gb300_pw_density_rs2pw / grid_gb300_pw_potential_pw2rs.

Only tests/ may import this module.  It restates, for replicated grids and
the default interpolation (pw_interp):
  * density_rs2pw  (src/pw_env/rs_pw_interface.F:64-136): every level grid to
    G space (forward FFT divided by the number of points,
    src/pw/fft_tools.F:394-397), the coefficients summed on the finest grid's
    frequencies (pw_axpy between grids that reference each other,
    src/pw/pw_methods.F:748-925), back to real space without scaling;
  * potential_pw2rs (:151-228): the finest level copies the potential;
    coarser levels take its G-space coefficients at their frequencies
    (pw_copy), transform back and scale by dvol(level) / dvol(finest).
  * poisson: the periodic Hartree solve in G space
    (src/pw/pw_poisson_types.F:316-320, influence function 4 pi / |G|^2 with
    G = 0 set to zero; src/pw/pw_poisson_methods.F:363-367, the Hartree
    energy 0.5 * pw_integral_ab(rho_G, v_G) = 0.5 Omega sum conj(rho_G) v_G).
A grid of n points holds the frequencies -n/2 .. n/2 - 1
(src/pw/pw_grid_info.F:247-254).  Grids are [nz][ny][nx] arrays (x
fastest), given flat or shaped.
"""
from __future__ import annotations

import numpy as np


def _freq_index(n_coarse: int, n_fine: int) -> np.ndarray:
    """Fine-grid array index of every array index of a coarse grid."""
    a = np.arange(n_coarse)
    f = np.where(a < (n_coarse + 1) // 2, a, a - n_coarse)
    return np.where(f >= 0, f, f + n_fine)


def _maps(coarse, fine):
    # numpy axes: 0 = z, 1 = y, 2 = x; shapes given as (nx, ny, nz)
    return np.ix_(_freq_index(coarse[2], fine[2]), _freq_index(coarse[1], fine[1]),
                  _freq_index(coarse[0], fine[0]))


def density_rs2pw(npts, rs_grids):
    """npts: [(nx, ny, nz)] finest first; rs_grids: level grids.  Returns
    (rho on the finest grid, its G-space coefficients [nz][ny][nx])."""
    fine = tuple(npts[0])
    g = np.zeros((fine[2], fine[1], fine[0]), np.complex128)
    for n, r in zip(npts, rs_grids):
        r = np.asarray(r, np.float64).reshape(n[2], n[1], n[0])
        c = np.fft.fftn(r) / r.size
        g[_maps(n, fine)] += c
    rho = np.real(np.fft.ifftn(g) * g.size)
    return rho, g


def potential_pw2rs(npts, v_rspace):
    """The potential on every level grid from the potential on the finest."""
    fine = tuple(npts[0])
    v = np.asarray(v_rspace, np.float64).reshape(fine[2], fine[1], fine[0])
    g = np.fft.fftn(v) / v.size
    out = [v.copy()]
    for n in npts[1:]:
        c = g[_maps(n, fine)]
        r = np.real(np.fft.ifftn(c) * c.size)
        out.append(r * (v.size / r.size))
    return out


def cell_of(dh, npts):
    """hmat (columns: the cell vectors) of a grid with spacing matrix dh (row
    d: the step along lattice vector d) and npts = (nx, ny, nz) points."""
    dh = np.asarray(dh, np.float64).reshape(3, 3)
    return np.stack([npts[d] * dh[d] for d in range(3)], axis=1)


def g_vectors(dh, npts):
    """Cartesian G vectors [nz][ny][nx][3] of the grid's frequencies:
    G = 2 pi sum_d f_d b_d, b_d the rows of inv(hmat) (b_d . a_e = delta)."""
    hinv = np.linalg.inv(cell_of(dh, npts))
    f = [np.where(np.arange(n) < (n + 1) // 2, np.arange(n), np.arange(n) - n) for n in npts]
    fz, fy, fx = np.meshgrid(f[2], f[1], f[0], indexing="ij")
    return 2.0 * np.pi * (fx[..., None] * hinv[0] + fy[..., None] * hinv[1]
                          + fz[..., None] * hinv[2])


def poisson(rho_g, dh, npts):
    """v(G) = 4 pi rho(G) / |G|^2 (zero at G = 0) and the Hartree energy
    0.5 Omega sum conj(rho(G)) v(G)."""
    g = g_vectors(dh, npts)
    g2 = (g ** 2).sum(-1)
    rho_g = np.asarray(rho_g, np.complex128).reshape(g2.shape)
    inf = np.zeros_like(g2)
    nz = g2 > 0
    inf[nz] = 4.0 * np.pi / g2[nz]
    v = rho_g * inf
    omega = abs(np.linalg.det(cell_of(dh, npts)))
    e = 0.5 * omega * float(np.real(np.sum(np.conj(rho_g) * v)))
    return v, e

