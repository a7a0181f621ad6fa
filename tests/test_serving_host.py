"""Host logic of the serving and batched drivers (no GPU): workload generators, footprint
estimates, the per-request precision policy and the prewarm shapes."""

from math import comb

import numpy as np


def test_poisson_stream_is_seeded_and_weighted():
    from forte2_gb300.serve import poisson_stream

    a = poisson_stream(2000, rate=200.0, seed=5)
    b = poisson_stream(2000, rate=200.0, seed=5)
    assert [(r.arrival, r.norb, r.multiplicity, r.nroot, r.iseed) for r in a] == \
           [(r.arrival, r.norb, r.multiplicity, r.nroot, r.iseed) for r in b]
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) > 0)
    assert abs(len(a) / t[-1] - 200.0) < 20.0  # mean rate
    counts = {n: sum(r.norb == n for r in a) for n in (6, 8, 10)}
    # weight proportional to 1 / Ndet: (6e,6o) is C(8,4)^2 / C(6,3)^2 = 12.25 times as likely as (8e,8o)
    assert 8 < counts[6] / max(counts[8], 1) < 18
    assert {r.multiplicity for r in a} == {1, 3} and {r.nroot for r in a} == {1, 2, 3}


def test_request_precision_policy():
    from forte2_gb300.serve import Request, request_precision

    small = Request(0, 0.0, 8, 1, 1, 1)
    large = Request(1, 0.0, 12, 1, 1, 1)
    assert comb(12, 6) ** 2 >= 200_000 > comb(8, 4) ** 2
    assert request_precision(small, "mixed") == "fp64"
    assert request_precision(large, "mixed") == "mixed"
    assert request_precision(large, "fp64") == "fp64"
    assert request_precision(small, "mixed", mixed_min_ndet=0) == "mixed"


def test_footprint_grows_with_space_and_roots():
    from forte2_gb300.batch import footprint_bytes

    f = [footprint_bytes(n, n // 2, n // 2, 2) for n in (6, 8, 10, 12, 14, 16)]
    assert all(x < y for x, y in zip(f, f[1:]))
    assert footprint_bytes(12, 6, 6, 3) > footprint_bytes(12, 6, 6, 1)
    assert footprint_bytes(16, 8, 8, 1) > 10 * 2**30  # CAS(16,16) needs tens of GB


def test_batched_instances_and_prewarm_shapes():
    from forte2_gb300.batch import batched_instances
    from forte2_gb300.serve import default_prewarm

    inst = batched_instances(64, seed=4000)
    assert len(inst) == 64 and {x["norb"] for x in inst} <= {8, 10, 12}
    assert all(x["na"] == x["nb"] == x["norb"] // 2 and 1 <= x["nroot"] <= 4 for x in inst)
    shapes = default_prewarm()
    assert len(shapes) == 18 and sum(c for *_, c in shapes) == 6 * (16 + 6 + 2)


def test_server_solvers_keep_allocating_fp32_options_off():
    from forte2_gb300.serve import Request, SolverPool

    pool = SolverPool("mixed", 1e-10)
    assert pool.variants(Request(0, 0.0, 12, 1, 1, 1)) == {"tma_b": 0, "dense_same_spin": 0}
    assert pool.variants(Request(1, 0.0, 8, 1, 1, 1)) is None  # FP64 below the mixed threshold
    assert SolverPool("fp64", 1e-10).variants(Request(2, 0.0, 12, 1, 1, 1)) is None


class _FakeBuilder:
    """The two calls the autotuner's candidate list makes, recorded."""

    def __init__(self, dense_ok=True):
        self.calls = []
        self.dense_ok = dense_ok

    def set_tensor_cores(self, on=True):
        return True

    def set_variant(self, name, value):
        if name == "dense_same_spin" and value and not self.dense_ok:
            raise ValueError("dense same-spin GEMMs need at most 4096 strings per spin")
        self.calls.append((name, value))


def test_autotune_candidates_honour_fixed_variants():
    from forte2_gb300.autotune import candidates

    sb = _FakeBuilder()
    full = candidates(sb, "fp32")
    assert len(full) == 16 and {c["dense_same_spin"] for c in full} == {0, 1}
    sb = _FakeBuilder()
    fixed = candidates(sb, "fp32", {"tma_b": 0, "dense_same_spin": 0})
    assert len(fixed) == 8
    assert all(c["tma_b"] == 0 and c["dense_same_spin"] == 0 for c in fixed)
    assert ("dense_same_spin", 1) not in sb.calls  # a fixed option is never switched on to probe it
    sb = _FakeBuilder(dense_ok=False)
    assert all("dense_same_spin" not in c for c in candidates(sb, "fp32"))
    assert len(candidates(_FakeBuilder(), "fp64")) == 4
