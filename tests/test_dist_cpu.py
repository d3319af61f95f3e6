"""Multi-process path of bench.py on CPU (gloo, world size 2): each rank times
its own batch, the job time is the slowest rank's, the rate counts every
rank's units, and the reference arm runs on rank 0 only."""

import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, w)  # rank 1 is slower
        q.put((r, w, local, ms, bench.job_rate(32, w, ms)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29611
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, local, ms, rate in out:
        assert w == 2 and local == r
        assert ms == 15.0
        assert rate == pytest.approx(32 * 2 / 0.015)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup = 1, 1

    assert bench.reference_arm(Args()) is None
    assert capsys.readouterr().out == ""


def _grad_worker(rank, world, port, q):
    """One gloo rank: the oracle's partial gradient of its bands (16^2 grid,
    4 bands), summed over ranks by the product's sharded reduction."""
    sys.path.insert(0, ROOT)
    from oracle import adjoint as o_adj
    from optics_studio_gb300 import inverse as inv
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        phi, bands, w = _grad_case()

        def partial(idx):
            rend, merit = _oracle_setup([bands[i] for i in idx], w)
            g = o_adj.grid_gradient(rend, phi.reshape(-1), merit)
            val = merit.evaluate(rend.render(phi.reshape(-1)))
            return {k: torch.from_numpy(v.copy()) for k, v in g.items()}, val

        grads, val = inv.grid_gradient_sharded(partial, len(bands))
        q.put((rank, inv.shard_bands(len(bands), rank, world),
               {k: v.numpy() for k, v in grads.items()}, val))
    finally:
        dist.destroy_process_group()


def _grad_case():
    import math
    import numpy as np
    n = 16
    phi = np.random.default_rng(3).uniform(0.0, 2 * math.pi, (n, n))
    bands = [500e-9, 530e-9, 560e-9, 600e-9]
    w = np.zeros((n, n))
    w[5:8, 5:8] = 1.0
    w[9:11, 8:12] = 0.5
    return phi, bands, w


def _oracle_setup(bands, w):
    from oracle import asm as o_asm, carrier as o_car, element as o_el
    from oracle import field as o_field, merit as o_merit, observe as o_obs
    import math
    n, d = 16, 4e-6

    def design(v, lam):
        dz = o_car.Design()
        dz.push(o_el.PhaseMask.sampled(v, (n, n), (d, d)), 0.3e-3)
        return dz

    car = o_car.Carrier.analytic(n * n, 0.0, 2 * math.pi, design)
    src = lambda x0, y0, lam: o_field.gaussian(20e-6, 1.0, (x0, y0), 0.0, lam, n, n, d, d)
    rend = o_obs.Renderer(car, src, bands=list(bands), asm_cfg=o_asm.AsmConfig())
    return rend, o_merit.WeightedSpotEfficiency(w, [1.0] * len(bands))


def test_band_sharded_gradient_sum_matches_one_rank():
    """The one exchange of the inverse-design step: bands split over two gloo
    ranks, partial gradients summed by one all-reduce, equal (to rounding of
    the summation order) to the gradient of all bands on one rank."""
    import numpy as np
    from oracle import adjoint as o_adj
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_grad_worker, args=(r, 2, 29617, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    phi, bands, w = _grad_case()
    rend, merit = _oracle_setup(bands, w)
    want = o_adj.grid_gradient(rend, phi.reshape(-1), merit)
    want_val = merit.evaluate(rend.render(phi.reshape(-1)))
    assert out[0][1] == [0, 2] and out[1][1] == [1, 3]
    for rank, idx, grads, val in out:
        assert sorted(grads) == sorted(want)
        for k in want:
            np.testing.assert_allclose(grads[k], want[k], rtol=1e-12,
                                       atol=1e-12 * np.abs(want[k]).max())
        assert val == pytest.approx(want_val, rel=1e-12)
