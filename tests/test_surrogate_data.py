"""The surrogate's randomized training runs (CPU only): the parameters drawn
around the target workload, and which sources each run carries."""
import numpy as np

from swap_gb300.hybrid import config
from swap_gb300.surrogate_data import run_config


def test_runs_keep_the_workload_and_draw_their_upstream_state():
    base = config(1)
    rng = np.random.default_rng(3)
    va = base.b0 / np.sqrt(base.n0)
    kinds = set()
    for r in range(64):
        cfg = run_config(base, rng, (32, 32, 32), r)
        assert cfg.cells == (32, 32, 32)
        assert (cfg.ppc, cfg.b0, cfg.dt, cfg.ntsub) == (base.ppc, base.b0, base.dt, base.ntsub)
        u = cfg.u[0] / va
        beta = (cfg.vth / va) ** 2
        assert 1.0 <= u <= 6.0 and 0.1 <= beta <= 2.0 and cfg.u[1:] == (0.0, 0.0)
        src = cfg.sources
        cloud, x_open = bool(src.get("cloud_N0")), bool(src.get("x_open"))
        kinds.add((cloud, x_open))
        if cloud:
            assert 2.0 <= src["cloud_r0"] <= 10.0 and src["cx_a"] == 1.0
            assert src["cloud_x"] == 17.0  # the box centre
        if x_open:
            assert src["inflow_ux"] == cfg.u[0] and src["inflow_vth"] == cfg.vth
        if not (cloud or x_open):
            assert src == {}
    # mixed: every combination of cloud and open x occurs
    assert kinds == {(False, False), (False, True), (True, False), (True, True)}


def test_unmixed_runs_all_carry_the_cloud_and_the_inflow():
    base = config(1)
    rng = np.random.default_rng(5)
    for r in range(16):
        src = run_config(base, rng, (32, 32, 32), r, mixed=False).sources
        assert src["cloud_N0"] == 1000.0 and src["x_open"] == 1


def test_runs_repeat_for_a_seed():
    base = config(1)
    a = [run_config(base, np.random.default_rng(9), (32, 32, 32), r) for r in range(1)]
    b = [run_config(base, np.random.default_rng(9), (32, 32, 32), r) for r in range(1)]
    assert a[0].u == b[0].u and a[0].vth == b[0].vth and a[0].seed == b[0].seed and a[0].sources == b[0].sources


def test_capacity_hint_covers_the_workloads_growth():
    """ni_max_hint: the load plus 10% for inflow and outflow, the cloud's new
    ions over the steps, and with charge exchange every ion that enters."""
    periodic = config(0)
    assert periodic.ni_max_hint() == periodic.n_particles  # no sources: no change
    c3 = config(3)
    n = c3.n_particles
    cloud = c3.cloud_ions_per_step()
    assert cloud > 0
    h = c3.ni_max_hint(200)
    assert h >= int(n * 1.10 + 1.1 * cloud * 200)
    # 200 steps of the 512x256x256 run grew the count 1.7% (FP64 drop-in)
    assert h > 1.017 * n
    src = dict(c3.sources)
    src.update(cx_a=0.0, cx_b=0.0)
    no_cx = config(3, sources=src)
    assert no_cx.ni_max_hint(200) < h  # with exchange, the entering ions stay
