"""CPU checks of the plane-wave transfer oracle (oracle/pw_oracle.py), the
restatement of CP2K's density_rs2pw / potential_pw2rs
(src/pw_env/rs_pw_interface.F:64-228) that the GPU transfer is tested
against."""
import numpy as np

from oracle import pw_oracle as P

NPTS = [(24, 20, 18), (18, 15, 12), (12, 10, 9)]  # even and odd sizes


def _rand(n, rng):
    return rng.uniform(-1.0, 1.0, size=n[0] * n[1] * n[2])


def test_adjointness():
    """<density_rs2pw(rs), V> = sum_l <rs_l, potential_pw2rs(V)_l>: the two
    transfers are adjoint, so Tr(V rho) does not depend on the side of the
    transfer it is taken on."""
    rng = np.random.default_rng(1)
    rs = [_rand(n, rng) for n in NPTS]
    rho, _ = P.density_rs2pw(NPTS, rs)
    V = _rand(NPTS[0], rng)
    Vl = P.potential_pw2rs(NPTS, V)
    lhs = float((rho.ravel() * V).sum())
    rhs = sum(float((r * v.ravel()).sum()) for r, v in zip(rs, Vl))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


def test_single_level_is_identity():
    rng = np.random.default_rng(2)
    rs = _rand(NPTS[0], rng)
    rho, g = P.density_rs2pw(NPTS[:1], [rs])
    assert np.abs(rho.ravel() - rs).max() < 1e-14
    assert abs(g[0, 0, 0].real - rs.mean()) < 1e-15


def test_band_limited_potential_is_sampled():
    """A potential with frequencies inside every level's box arrives on each
    coarse level as its samples there, times dvol(level) / dvol(finest)."""
    fine = NPTS[0]
    z, y, x = np.meshgrid(*(np.arange(fine[d]) / fine[d] for d in (2, 1, 0)), indexing="ij")
    V = np.cos(2 * np.pi * (2 * x + y)) + 0.5 * np.sin(2 * np.pi * (x - 3 * z))
    Vl = P.potential_pw2rs(NPTS, V)
    for n, v in zip(NPTS[1:], Vl[1:]):
        zc, yc, xc = np.meshgrid(*(np.arange(n[d]) / n[d] for d in (2, 1, 0)), indexing="ij")
        want = np.cos(2 * np.pi * (2 * xc + yc)) + 0.5 * np.sin(2 * np.pi * (xc - 3 * zc))
        scale = (fine[0] * fine[1] * fine[2]) / (n[0] * n[1] * n[2])
        assert np.abs(v - scale * want).max() < 1e-12
