"""Known-answer tests of the CPU oracle (the reference ships none besides
b0.dat).  Each checks a property the reference algorithm has exactly or to
roundoff."""
import numpy as np

from helpers import Host, oracle, small


def test_rotation_is_exact_cayley():
    """E = 0, uniform B: get_vplus_vminus (gutsp.f:382-397) rotates v about
    B by theta with tan(theta/2) = B'dt/2 and keeps |v|."""
    h = Host(small(), ni_max=1, load=False)
    h.ni_tot[0] = 1
    h.xp[0] = (3.3, 2.7, 4.1)
    h.vp[0] = (0.7, -0.2, 0.4)
    o = oracle(h)
    o.btc[...] = 0.0
    o.btc[..., 2] = 1.5  # B' = mrat*B with mrat = 1
    o.get_interp_weights(o.xp)
    o.Ep[...] = 0.0
    o.get_vplus_vminus(o.Ep, o.btc, o.vp, o.vplus, o.vminus)
    v0, v1 = o.vp[0], o.vplus[0]
    assert abs(np.linalg.norm(v1) - np.linalg.norm(v0)) < 1e-15
    assert abs(v1[2] - v0[2]) < 1e-15
    theta = np.arctan2(v0[0] * v1[1] - v0[1] * v1[0], v0[0] * v1[0] + v0[1] * v1[1])
    dt = h.cfg.dt
    assert abs(np.tan(-theta / 2) - 1.5 * dt / 2) < 1e-14


def test_exb_drift_velocity_is_a_fixed_point():
    """A particle moving at the E x B velocity with E = -u x B keeps v = u
    through the half kick, rotation and half kick (gutsp.f:302-446)."""
    h = Host(small(), ni_max=3, load=False)
    h.ni_tot[0] = 3
    h.xp[:] = [(2.2, 3.1, 1.9), (5.5, 4.4, 6.1), (7.9, 1.2, 3.3)]
    u = np.array([1.3, -0.4, 0.25])
    h.vp[:] = u
    o = oracle(h)
    B = np.array([0.2, -0.3, 1.1])
    o.btc[...] = B
    o.get_interp_weights(o.xp)
    E = -np.cross(u, B)
    o.Ep[:] = E
    o.get_vplus_vminus(o.Ep, o.btc, o.vp, o.vplus, o.vminus)
    o.get_vp_final(o.Ep, o.vp, o.vp1, o.vplus)
    assert np.max(np.abs(o.vp - u)) < 1e-15


def test_cell_index_on_nodes():
    """x exactly on node i: the strict '>' search gives i-1
    (gutsp.f:1396-1401); y exactly on node j: floor gives j (gutsp.f:1404)."""
    h = Host(small(), ni_max=2, load=False)
    h.ni_tot[0] = 2
    h.xp[0] = (h.coords.qx[4], h.coords.qy[3], h.coords.qz[2])  # nodes 5, 4, 3 (1-based)
    h.xp[1] = (h.coords.qx[4] + 1e-12, h.coords.qy[3] - 1e-12, h.coords.qz[2] + 1e-12)
    o = oracle(h)
    o.get_interp_weights(o.xp)
    ijk = o.ijkp()
    assert tuple(ijk[0]) == (4, 4, 2)
    assert tuple(ijk[1]) == (5, 3, 3)


def test_uniform_lattice_density_is_exact_after_fold():
    """Particles at cell centres deposit 1/8 to each corner; with ppc per
    cell and beta = ppc the folded density (gutsp.f:1496-1498) is exactly n0
    everywhere, ghosts included (periodic_scalar)."""
    cfg = small(ppc=4)  # beta = 4: every term 1/32 is exact in binary
    h = Host(cfg, load=False)
    nx, ny, nz = cfg.nodes
    ii, jj, kk = np.meshgrid(np.arange(nx - 2), np.arange(ny - 2), np.arange(nz - 2), indexing="ij")
    centres = np.stack([h.coords.qx[ii.ravel()] + 0.5, h.coords.qy[jj.ravel()] + 0.5,
                        h.coords.qz[kk.ravel()] + 0.5], axis=1)
    pts = np.repeat(centres, cfg.ppc, axis=0)
    h.xp[: len(pts)] = pts
    h.ni_tot[0] = len(pts)
    o = oracle(h)
    o.get_interp_weights(o.xp)
    o.update_np(o.np)
    assert np.all(o.np == 1.0)


def test_cold_beam_in_uniform_B_is_stationary():
    """vth = 0, u = (2,0,0), uniform B: up = u, aj = 0, E = -u x B is
    uniform, curl E = 0, so B and v stay put (to roundoff)."""
    cfg = small(vth=0.0, ppc=2)
    h = Host(cfg)
    o = oracle(h)
    for _ in range(3):
        o.ion_step()
    n = int(o.ni_tot[0])
    assert np.max(np.abs(o.b1 - o.b0)) < 1e-13
    assert np.max(np.abs(o.vp[:n] - np.array([2.0, 0.0, 0.0]))) < 1e-13
    assert np.max(np.abs(o.up[..., 0] - 2.0)) < 1e-13


def test_div_B_is_preserved():
    """curlE uses forward differences (gutsf.f:288-299); the forward-difference
    divergence of any discrete curl vanishes, so B updates keep div B at
    roundoff while B itself evolves."""
    cfg = small(ppc=8)
    h = Host(cfg)
    o = oracle(h)
    for _ in range(4):
        o.ion_step()
    assert np.max(np.abs(o.b1 - o.b0)) > 1e-3
    assert o.max_abs_divB(o.b1) < 1e-12


def test_periodic_wrap_invariants():
    """move_ion_half (gutsp.f:490-510) wraps into (q(1), q(n-1)]."""
    cfg = small()
    h = Host(cfg, ni_max=4, load=False)
    q = h.coords
    L = q.qx[-2] - q.qx[0]
    eps = 0.01
    h.ni_tot[0] = 4
    h.xp[0] = (q.qx[-2] - eps, 3.0, 3.0)
    h.xp[1] = (q.qx[0] + eps, 3.0, 3.0)
    h.xp[2] = (3.0, q.qy[-2], 3.0)
    h.xp[3] = (3.0, 3.0, q.qz[0] + 1e-9)
    dth = cfg.dt / 2
    h.vp[0] = (2 * eps / dth, 0, 0)
    h.vp[1] = (-2 * eps / dth, 0, 0)
    h.vp[2] = (0, 0.0, 0)
    h.vp[3] = (0, 0, -2e-9 / dth)
    o = oracle(h)
    o.move_ion_half(o.xp, o.vp, o.vp1, o.input_p)
    assert abs(o.xp[0, 0] - (q.qx[0] + eps)) < 1e-12
    assert abs(o.xp[1, 0] - (q.qx[-2] - eps)) < 1e-12
    assert o.xp[2, 1] == q.qy[-2]  # on the upper face stays (q(1), q(n-1)]
    assert q.qz[-2] - 1e-8 < o.xp[3, 2] <= q.qz[-2]
    assert L == (cfg.nodes[0] - 2) * 1.0


def _courant_reference(bt, np_, alpha, dx, dtsub, ntf):
    # check_time_step (gutsf.f:1782-1806) restated independently in numpy
    nx, ny, nz = np_.shape
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                ak = 2.0 / dx
                btot = np.sqrt(bt[i, j, k, 0] ** 2 + bt[i, j, k, 1] ** 2 + bt[i, j, k, 2] ** 2)
                a1 = ak ** 2 * btot / (alpha * np_[i, j, k])
                a2 = (ak * btot) ** 2 / (alpha * np_[i, j, k])
                womega = 0.5 * (a1 + np.sqrt(a1 ** 2 + 4 * a2))
                deltat = dx / (womega / ak)
                if deltat <= 2.0 * dtsub:
                    dtsub /= 2.0
                    ntf *= 2.0
    return dtsub, ntf


def test_courant_rule_halves_per_violating_node():
    cfg = small(dt=5.0, cells=(4, 3, 3))  # dtsub = 0.5: far past the whistler limit
    h = Host(cfg)
    o = oracle(h)
    o.get_interp_weights(o.xp)
    o.update_np(o.np)
    rng = np.random.default_rng(1)
    o.bt[...] = o.b0 * (1 + 0.5 * rng.random(o.b0.shape))
    got = o.check_time_step(o.bt, o.np, cfg.dt / cfg.ntsub, float(cfg.ntsub))
    want = _courant_reference(o.bt, o.np, cfg.alpha, 1.0, cfg.dt / cfg.ntsub, float(cfg.ntsub))
    assert got == want and got[1] > cfg.ntsub


def test_fp32_and_fp64_oracles_agree_over_a_few_steps():
    cfg = small(ppc=8)
    h = Host(cfg)
    for a in (h.xp, h.vp, h.vp1):
        a[...] = a.astype(np.float32)
    o64 = oracle(h, "f64")
    o32 = oracle(h, "f32")
    for _ in range(3):
        o64.ion_step()
        o32.ion_step()
    d = np.linalg.norm(o32.b1 - o64.b1) / np.linalg.norm(o64.b1)
    assert 0 < d < 1e-5
    n = int(h.ni_tot[0])
    assert np.max(np.abs(o32.xp[:n] - o64.xp[:n])) < 1e-4


def test_counting_sort_is_stable_and_complete():
    cfg = small(ppc=5)
    h = Host(cfg)
    o = oracle(h)
    rng = np.random.default_rng(3)
    n = int(o.ni_tot[0])
    p = rng.permutation(n)
    o.xp[:n] = o.xp[p]
    o.get_interp_weights(o.xp)
    perm, counts = o.sort_perm(n)
    ijk = o.ijkp()[:n]
    nx, ny, _ = cfg.nodes
    key = (ijk[:, 0] - 1) + nx * ((ijk[:, 1] - 1) + ny * (ijk[:, 2] - 1))
    ks = key[perm]
    assert np.all(np.diff(ks) >= 0)
    for c in np.unique(ks):  # stable: original order inside a cell
        assert np.all(np.diff(perm[ks == c]) > 0)
    assert counts.sum() == n and np.array_equal(np.bincount(key, minlength=counts.size), counts)
    assert np.all(counts[np.unique(key)] == cfg.ppc)
