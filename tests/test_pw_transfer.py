"""GPU: the device-resident plane-wave transfer of the level grids
(grid_gb300_pw_density_rs2pw / grid_gb300_pw_potential_pw2rs, CP2K's
density_rs2pw / potential_pw2rs of src/pw_env/rs_pw_interface.F:64-228)
against the numpy restatement (oracle/pw_oracle.py) on the same seeded grids,
max |d| / max |ref| <= 1e-12 (FP64 FFTs of both); at the 512-atom workload's
level sizes through the size-independent adjointness of the two transfers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("npts", [
    [(24, 20, 18), (18, 15, 12), (12, 10, 9)],
    [(40, 40, 40), (30, 30, 30), (20, 20, 20), (15, 15, 15)],
])
def test_pw_transfer_matches_oracle(npts):
    import torch
    from cp2k_gb300 import grid as G
    from oracle import pw_oracle as P
    rng = np.random.default_rng(3)
    rs_h = [rng.uniform(-1, 1, size=n[0] * n[1] * n[2]) for n in npts]
    V_h = rng.uniform(-1, 1, size=npts[0][0] * npts[0][1] * npts[0][2])
    rho_o, g_o = P.density_rs2pw(npts, rs_h)
    Vl_o = P.potential_pw2rs(npts, V_h)
    dev = torch.device("cuda", 0)
    pw = G.PwTransfer(npts)
    rs = [torch.tensor(r, device=dev) for r in rs_h]
    rho = torch.empty(rs_h[0].size, dtype=torch.float64, device=dev)
    g = torch.empty(2 * rs_h[0].size, dtype=torch.float64, device=dev)
    pw.density_rs2pw(rs, rho, g)
    V = torch.tensor(V_h, device=dev)
    Vl = [torch.empty(r.size, dtype=torch.float64, device=dev) for r in rs_h]
    pw.potential_pw2rs(V, Vl)
    torch.cuda.synchronize()
    err = lambda a, b: float(np.abs(a - b).max()) / float(np.abs(b).max())
    assert err(rho.cpu().numpy(), rho_o.ravel()) < 1e-12
    gc = g.cpu().numpy().view(np.complex128)
    assert err(gc, g_o.ravel()) < 1e-12
    for a, b in zip(Vl, Vl_o):
        assert err(a.cpu().numpy(), b.ravel()) < 1e-12
    pw.close()


def test_pw_transfer_adjoint_at_full_size():
    """512-atom workload levels 216^3 .. 54^3: <rho, V> on the finest grid
    equals sum over levels <rs_l, V_l>, and collocate -> rs2pw -> pw2rs ->
    integrate stays on the device."""
    import torch
    from cp2k_gb300 import grid as G
    npts = [(n, n, n) for n in (216, 152, 108, 76, 54)]
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev).manual_seed(5)
    rs = [torch.rand(n[0] ** 3, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
          for n in npts]
    V = torch.rand(216 ** 3, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
    pw = G.PwTransfer(npts)
    rho = torch.empty(216 ** 3, dtype=torch.float64, device=dev)
    pw.density_rs2pw(rs, rho)
    Vl = [torch.empty_like(r) for r in rs]
    pw.potential_pw2rs(V, Vl)
    lhs = float((rho * V).sum())
    rhs = sum(float((r * v).sum()) for r, v in zip(rs, Vl))
    assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(lhs))
    pw.close()
