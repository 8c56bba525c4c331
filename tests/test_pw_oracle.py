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


def test_g_vectors_are_the_cells_reciprocal_lattice():
    """On a triclinic cell every G of the grid's frequencies gives a plane
    wave with the cell's periods: G . a_d = 2 pi f_d."""
    dh = np.array([[0.20, 0.00, 0.00], [0.05, 0.19, 0.00], [-0.03, 0.04, 0.21]])
    npts = (12, 10, 9)
    g = P.g_vectors(dh, npts)
    h = P.cell_of(dh, npts)
    f = [np.where(np.arange(n) < (n + 1) // 2, np.arange(n), np.arange(n) - n) for n in npts]
    fz, fy, fx = np.meshgrid(f[2], f[1], f[0], indexing="ij")
    for d, fd in enumerate((fx, fy, fz)):
        assert np.allclose(g @ h[:, d], 2 * np.pi * fd, atol=1e-10)


def test_poisson_against_finite_differences():
    """On an orthorhombic box the potential of a smooth, neutral charge
    satisfies -Laplacian(v) = 4 pi rho (second-order finite differences, to
    their truncation error), and the Hartree energy is 0.5 int v rho."""
    n, h = (48, 40, 44), (0.25, 0.3, 0.28)
    dh = np.diag(h)
    L = [n[d] * h[d] for d in range(3)]
    z, y, x = np.meshgrid(*[np.arange(n[d]) * h[d] for d in (2, 1, 0)], indexing="ij")
    def gauss(c, a):
        r2 = sum(((q - c[i] + L[i] / 2) % L[i] - L[i] / 2) ** 2
                 for i, q in zip((0, 1, 2), (x, y, z)))
        return (a / np.pi) ** 1.5 * np.exp(-a * r2)
    rho = gauss((3.0, 5.0, 6.0), 1.5) - gauss((8.0, 6.0, 4.0), 0.8)  # neutral
    rho_g = np.fft.fftn(rho) / rho.size
    v_g, e = P.poisson(rho_g, dh, n)
    v = np.real(np.fft.ifftn(v_g) * v_g.size)
    lap = sum((np.roll(v, 1, ax) - 2 * v + np.roll(v, -1, ax)) / hh ** 2
              for ax, hh in ((2, h[0]), (1, h[1]), (0, h[2])))
    assert float(np.abs(-lap - 4 * np.pi * rho).max()) < 0.05 * float(np.abs(4 * np.pi * rho).max())
    dvol = h[0] * h[1] * h[2]
    assert abs(e - 0.5 * float((v * rho).sum()) * dvol) < 1e-10 * abs(e)
