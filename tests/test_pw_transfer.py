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


def test_pw_poisson_matches_oracle():
    """The periodic Hartree solve on a triclinic cell against the numpy
    restatement: v(G), v in real space and the Hartree energy to 1e-12."""
    import torch
    from cp2k_gb300 import grid as G
    from oracle import pw_oracle as P
    npts = [(24, 20, 18), (12, 10, 9)]
    dh = np.array([[0.20, 0.00, 0.00], [0.05, 0.19, 0.00], [-0.03, 0.04, 0.21]])
    rng = np.random.default_rng(11)
    rs_h = [rng.uniform(-1, 1, size=n[0] * n[1] * n[2]) for n in npts]
    _, g_o = P.density_rs2pw(npts, rs_h)
    v_o, e_o = P.poisson(g_o, dh, npts[0])
    vr_o = np.real(np.fft.ifftn(v_o) * v_o.size)
    dev = torch.device("cuda", 0)
    pw = G.PwTransfer(npts)
    rs = [torch.tensor(r, device=dev) for r in rs_h]
    n0 = rs_h[0].size
    g = torch.empty(2 * n0, dtype=torch.float64, device=dev)
    pw.density_rs2pw(rs, None, g)
    v = torch.empty(2 * n0, dtype=torch.float64, device=dev)
    vr = torch.empty(n0, dtype=torch.float64, device=dev)
    e = pw.poisson(dh, g, v, vr, energy=True)
    err = lambda a, b: float(np.abs(a - b).max()) / float(np.abs(b).max())
    assert err(v.cpu().numpy().view(np.complex128), v_o.ravel()) < 1e-12
    assert err(vr.cpu().numpy(), vr_o.ravel()) < 1e-12
    assert abs(e - e_o) <= 1e-12 * abs(e_o)
    pw.poisson(dh, g, g)  # in place, no energy
    torch.cuda.synchronize()
    assert err(g.cpu().numpy().view(np.complex128), v_o.ravel()) < 1e-12
    pw.close()


def test_hartree_step_on_device():
    """One Hartree step of the 64-atom workload kept on the device:
    collocate -> density_rs2pw -> Poisson -> potential_pw2rs -> integrate,
    against the same chain on the host with the oracle (CP2K's REF
    restatement) and the numpy transfer and Poisson: Hartree energy and hab
    within 1e-10 (FP64 throughout; FFT rounding)."""
    import torch
    from cp2k_gb300 import grid as G
    from cp2k_gb300 import workload as W
    from oracle import oracle as O
    from oracle import pw_oracle as P
    inp = W.config("c1_64atoms", scale=0.3, seed=9)
    pab = W.density_blocks(inp)
    npts = [tuple(int(x) for x in n) for n in inp.npts_local]
    dh = np.asarray(inp.dh[0], np.float64).reshape(3, 3)
    # host chain
    ot = O.OracleTaskList(inp)
    rho_l = ot.collocate(100, pab)
    _, g_h = P.density_rs2pw(npts, [r.ravel() for r in rho_l])
    v_h, e_h = P.poisson(g_h, dh, npts[0])
    vr_h = np.real(np.fft.ifftn(v_h) * v_h.size)
    V_l = P.potential_pw2rs(npts, vr_h.ravel())
    hab_h, _, _ = ot.integrate([v.ravel() for v in V_l])
    ot.close()
    # device chain
    dev = torch.device("cuda", 0)
    tl = G.GridTaskList(inp, precision=G.FP64)
    pw = G.PwTransfer(npts)
    pab_d = torch.tensor(pab, device=dev)
    grids = [torch.empty(int(np.prod(n)), dtype=torch.float64, device=dev) for n in npts]
    n0 = int(np.prod(npts[0]))
    g = torch.empty(2 * n0, dtype=torch.float64, device=dev)
    vr = torch.empty(n0, dtype=torch.float64, device=dev)
    hab = torch.empty(inp.buffer_size, dtype=torch.float64, device=dev)
    st = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(st):
        tl.collocate_device(100, pab_d, grids, stream=st)
        pw.density_rs2pw(grids, None, g, stream=st)
        e = pw.poisson(dh, g, g, vr, energy=True, stream=st)
        pw.potential_pw2rs(vr, grids, stream=st)
        tl.integrate_device(grids, hab, stream=st)
    torch.cuda.synchronize()
    assert abs(e - e_h) <= 1e-10 * abs(e_h)
    h = hab.cpu().numpy()
    assert float(np.abs(h - hab_h).max()) <= 1e-10 * max(1.0, float(np.abs(hab_h).max()))
    # the same potential on the level grids straight from v(G) (one FFT
    # fewer than the host chain's real-space round trip: the same 1e-10)
    lv = [torch.empty_like(x) for x in grids]
    pw.potential_g2rs(g, lv)
    torch.cuda.synchronize()
    for a, b in zip(lv, V_l):
        assert float(np.abs(a.cpu().numpy() - b.ravel()).max()) <= 1e-10 * float(np.abs(b).max())
    pw.close()
    tl.close()
