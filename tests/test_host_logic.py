"""Host-side logic: basis construction, seeded workloads, FLOP model, and the
multi-process (gloo, world size 2) replica split used for N > 1 GPUs."""
import math
import os
import socket

import numpy as np
import pytest

from gbhf import basis as B, molecules as M, replicas
from gbhf.flops_model import DEFERRED, F_ALG, F_KERNEL


def test_sp_shell_split_and_normalisation():
    cg = B.basis_for("O", "6-31g", "text")
    assert [c.funtype for c in cg] == ["S", "S", "Px", "Py", "Pz", "S", "Px", "Py", "Pz"]
    # normCoeff: c / sqrt(prod(2k-1)!! / (4a)^L * (pi/2a)^1.5)
    s = cg[0].primitives[0]
    a = 5484.6717
    assert s[1] == a
    assert s[0] == pytest.approx(0.0018311 / math.sqrt((math.pi / (2 * a)) ** 1.5), rel=1e-15)
    p = cg[2].primitives[0]
    a = 15.539616
    assert p[0] == pytest.approx(0.0708743 / math.sqrt(1 / (4 * a) * (math.pi / (2 * a)) ** 1.5), rel=1e-15)
    d = B.basis_for("O", "6-31g*", "text")
    assert [c.funtype for c in d[-6:]] == ["Dxx", "Dxy", "Dxz", "Dyy", "Dyz", "Dzz"]
    # Dxx carries (2*2-1)!! = 3 in the norm, Dxy does not
    assert d[-6].primitives[0][0] * math.sqrt(3) == pytest.approx(d[-5].primitives[0][0], rel=1e-14)


def test_shipped_basis_differs_only_in_sp_exponents():
    for el in ("H", "O"):
        sh = B.basis_for(el, "6-31g", "shipped")
        tx = B.basis_for(el, "6-31g", "text")
        assert len(sh) == len(tx)
        for a, b in zip(sh, tx):
            assert a.funtype == b.funtype
            ea = [p[1] for p in a.primitives]
            eb = [p[1] for p in b.primitives]
            if el == "O" and a is not sh[0]:
                assert ea == [1.0] * len(ea)
            else:
                assert ea == eb


def test_water_clusters_are_reproducible_and_physical():
    rng = np.random.default_rng(M.SEEDS["w16"])
    regenerated = M.water_cluster(16, rng)
    np.testing.assert_allclose(regenerated, M.cluster_coords("w16"), rtol=0, atol=1e-10)
    xyz = M.cluster_coords("w64") / B.ANGSTROM_TO_BOHR
    o = xyz[0::3]
    for w in range(64):
        r1 = np.linalg.norm(xyz[3 * w + 1] - xyz[3 * w])
        r2 = np.linalg.norm(xyz[3 * w + 2] - xyz[3 * w])
        ang = math.degrees(math.acos(np.dot(xyz[3 * w + 1] - xyz[3 * w], xyz[3 * w + 2] - xyz[3 * w]) / (r1 * r2)))
        assert r1 == pytest.approx(0.9572, abs=1e-9) and r2 == pytest.approx(0.9572, abs=1e-9)
        assert ang == pytest.approx(104.52, abs=1e-7)
    dist = np.linalg.norm(o[:, None] - o[None], axis=-1) + np.eye(64) * 10
    assert dist.min() >= 2.6 - 1e-9


def test_workload_sizes():
    assert B.n_basis(M.cluster_atoms("w16", "6-31g")) == 208
    assert B.n_basis(M.cluster_atoms("w8", "6-31g")) == 104
    assert B.n_basis(M.cluster_atoms("w64", "6-31g")) == 832
    batch = M.batch_workload()
    assert len(batch) == 256
    sizes = [len(m) // 3 for m in batch]
    assert min(sizes) >= 1 and max(sizes) <= 12
    for i in (0, 1):
        n = B.n_basis(batch[i])
        assert n == sizes[i] * (7 if i % 2 == 0 else 13)


def test_flop_model_table():
    sp = {k: F_ALG[k] for k in ("ssss", "psss", "psps", "ppss", "ppps", "pppp")}
    assert sp == {"ssss": 33, "psss": 98, "psps": 291, "ppss": 323, "ppps": 1004, "pppp": 3847}
    assert len(F_ALG) == 21 and F_ALG["dddd"] > F_ALG["dddp"] > F_ALG["pppp"]


def test_shard_balanced_and_complete():
    costs = [float(c) for c in np.random.default_rng(0).integers(1, 100, size=37)]
    parts = [replicas.shard(costs, 4, r) for r in range(4)]
    assert sorted(i for p in parts for i in p) == list(range(37))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    with pytest.raises(ValueError):
        replicas.shard(costs, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard(costs, world, rank)
    got = [None] * world
    dist.all_gather_object(got, mine)
    t = replicas.max_over_ranks(float(rank + 1))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got, t))


def test_gloo_two_ranks_replica_split():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    costs = [3.0, 1.0, 4.0, 1.0, 5.0, 9.0, 2.0]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, t in res:
        assert sorted(got[0] + got[1]) == list(range(len(costs)))
        assert not set(got[0]) & set(got[1])
        assert t == 2.0


def test_kernel_flop_model_of_the_deferred_classes():
    """The deferred-ket classes count the R recursion, Boys values, bra E
    products and the V contraction per primitive quartet: below F_alg, and
    F_KERNEL = F_alg for every other class."""
    assert set(DEFERRED) == {"psps", "ppss", "ppps"}
    assert (F_KERNEL["psps"], F_KERNEL["ppss"], F_KERNEL["ppps"]) == (165, 127, 302)
    for k, v in F_ALG.items():
        assert F_KERNEL[k] < v if k in DEFERRED else F_KERNEL[k] == v


def test_generated_headers_match_their_generators():
    """eri_gen.cuh and grad_gen.cuh are what gen_eri.py and gen_grad.py emit."""
    import importlib
    import sys
    from pathlib import Path
    csrc = Path(B.__file__).resolve().parents[1] / "csrc"
    sys.path.insert(0, str(csrc))
    try:
        for gen, out in (("gen_eri", "eri_gen.cuh"), ("gen_grad", "grad_gen.cuh")):
            mod = importlib.import_module(gen)
            assert mod.render() == (csrc / out).read_text(), out
    finally:
        sys.path.remove(str(csrc))


def test_bench_clock_sampler_keeps_samples_of_the_timed_region():
    """bench.py's ClockSampler: samples stamped inside the marked region (widened
    by one sampling period) count, earlier ones do not."""
    import datetime
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location("bench_mod", Path(__file__).resolve().parents[1] / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    c = bench.ClockSampler(0)
    now = datetime.datetime.now()
    c.t0, c.t1 = now, now + datetime.timedelta(seconds=0.3)

    def line(dt, mhz, power_cap):
        ts = (now + datetime.timedelta(seconds=dt)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return f"{ts}, 0, {mhz}, 2070, 900, 0x0, Not Active, Not Active, Not Active, {power_cap}"

    c.lines = [line(-1.0, 1000, "Not Active"), line(0.1, 2070, "Not Active"), line(0.45, 2060, "Active")]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2065.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
