"""The product's multi-rank exchange: two contexts on one GPU, each holding
half the ions (the reference's particle decomposition, maind.f:140), with
the moment deposits summed over the two through the exchange callback (the
MPI_ALLREDUCE of gutsp.f:1503,1812-1822), must reproduce the one-context run.

Each context runs in its own host thread; the callback is a host all-reduce:
it waits for its context's deposit, copies the sums to the host, meets the
other rank at a barrier, and writes the total back.  No kernel waits on
another: the ranks meet only on the host.  FP64 drop-in: the same fields to
rel-L2 1e-12 after three steps, with the open-x inflow given to rank 0 alone;
FP32 form: to its rounding (the two contexts sum the deposits in another
order).
"""
import threading

import numpy as np
import pytest

from conftest import rel_l2
from helpers import make_hybrid
from swap_gb300 import abi

pytestmark = pytest.mark.gpu


class _Dev:
    """A device array seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr, n, kind):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f4" if kind == 4 else "<f8",
                                         "data": (int(ptr), False), "strides": None, "version": 2}


class HostAllreduce:
    """An in-process all-reduce of n ranks, one host thread each."""

    def __init__(self, n):
        self.n = n
        self.bar = threading.Barrier(n, timeout=120)
        self.parts = [None] * n
        self.calls = [0] * n

    def callback(self, rank):
        import torch

        def fn(data, count, kind, stream):
            try:
                t = torch.as_tensor(_Dev(data, count, kind), device="cuda")
                torch.cuda.synchronize()  # the deposit queued on the library's stream is done
                self.parts[rank] = t.cpu()
                self.bar.wait()
                total = sum(self.parts)
                self.bar.wait()  # every rank has read every part
                t.copy_(total.to("cuda"))
                torch.cuda.synchronize()
                self.calls[rank] += 1
                return 0
            except Exception:
                self.bar.abort()
                return 1

        return fn


def _split(h, parts):
    """Keep every parts-th ion of h's load starting at each offset: one Hybrid per rank."""
    n = int(h.ni_tot[0])
    out = []
    for r in range(parts):
        hr = make_hybrid(**_KW)
        sel = np.arange(r, n, parts)
        for name in ("xp", "vp", "vp1"):
            a = getattr(hr, name)
            a[...] = 0
            a[: len(sel)] = getattr(h, name)[sel]
        for name in ("mrat", "beta_p"):
            a = getattr(hr, name)
            a[: len(sel)] = getattr(h, name)[sel]
        for name in ("b0", "b1", "b12", "b1p2", "bt", "np", "up", "nu"):
            getattr(hr, name)[...] = getattr(h, name)
        hr.ni_tot[0] = len(sel)
        hr.mark_host_dirty()
        out.append(hr)
    return out


_KW = dict(cells=(16, 8, 8), ppc=8, seed=17, db=0.02, extra=20000)


def _run_ranks(ranks, step):
    red = HostAllreduce(len(ranks))
    for r, h in enumerate(ranks):
        h.set_exchange(red.callback(r))
    errs = [None] * len(ranks)

    def work(r):
        try:
            step(ranks[r])
        except Exception as e:  # reported below
            errs[r] = e
            red.bar.abort()

    th = [threading.Thread(target=work, args=(r,)) for r in range(len(ranks))]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in th)
    assert errs == [None] * len(ranks), errs
    return red


def test_fp64_two_ranks_match_one_rank_with_inflow_on_rank0():
    cfg_src = dict(seed=5, x_open=1, inflow_vth=0.5, inflow_ux=2.0)
    one = make_hybrid(**_KW)
    ranks = _split(one, 2)
    one.set_sources(abi.make_sources(inflow_ppc=8, **cfg_src), 0)
    ranks[0].set_sources(abi.make_sources(inflow_ppc=8, **cfg_src), 0)
    ranks[1].set_sources(abi.make_sources(inflow_ppc=0, **cfg_src), 0)  # outflow only
    one.run(3)
    one.sync_to_host()
    red = _run_ranks(ranks, lambda h: h.run(3))
    assert red.calls == [3 * 6, 3 * 6]  # 2 density and 4 velocity deposits per step
    for h in ranks:
        h.sync_to_host()
    n = sum(int(h.ni_tot[0]) for h in ranks)
    assert n == int(one.ni_tot[0])
    for name in ("b1", "np", "up", "E"):
        for h in ranks:  # every rank holds the whole field
            assert rel_l2(getattr(h, name), getattr(one, name)) < 1e-12, name
    for h in ranks + [one]:
        h.close()


def test_f32_two_ranks_match_one_rank():
    one = make_hybrid(**_KW)
    ranks = _split(one, 2)
    one.f32_begin()
    e1 = one.f32_energy()
    one.f32_run(2)
    e_one = one.f32_energy()
    one.f32_end()
    one.sync_to_host()

    def step(h):
        h.f32_begin()
        h.f32_run(2)

    red = _run_ranks(ranks, step)
    assert red.calls == [2 * 3, 2 * 3]  # passes 1, 2 and 3 each deposit once
    ek = sum(h.f32_energy()[0] for h in ranks)  # kinetic: each rank's own ions
    for h in ranks:
        h.f32_end()
        h.sync_to_host()
    assert sum(int(h.ni_tot[0]) for h in ranks) == int(one.ni_tot[0])
    assert abs(ek - e_one[0]) / e_one[0] < 1e-5
    for h in ranks:
        assert rel_l2(h.b1, one.b1) < 1e-6
        assert rel_l2(h.b1 - h.b0, one.b1 - one.b0) < 1e-3
        assert rel_l2(h.np, one.np) < 1e-5
        assert rel_l2(h.up, one.up) < 1e-4
    assert e1[0] > 0
    for h in ranks + [one]:
        h.close()


def test_exchange_failure_is_reported():
    h = make_hybrid(cells=(8, 8, 8), ppc=2, seed=3)
    h.set_exchange(lambda data, count, kind, stream: 7)
    with pytest.raises(abi.SwapError) as ei:
        h.run(1)
    assert ei.value.code == 9  # SWAP_EEXCHANGE
    h.set_exchange(None)
    h.run(1)  # the context stays usable
    h.close()
