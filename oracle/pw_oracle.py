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
