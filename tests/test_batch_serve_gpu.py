"""Batched instances and the continuous-batching server: every result equals its solo solve."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_equals_loop(cuda):
    from forte2_gb300.batch import batched_instances, solve_batched, solve_loop

    inst = batched_instances(6, seed=11)
    for x in inst:  # keep the test quick: the smaller spaces of the batched workload
        x["norb"] = min(x["norb"], 8)
        x["na"] = x["nb"] = x["norb"] // 2
    loop, _ = solve_loop(inst)
    batched, _, rounds = solve_batched(inst, nstreams=4)
    assert rounds > 0
    for i in range(len(inst)):
        assert batched[i].converged and loop[i].converged
        np.testing.assert_allclose(batched[i].evals, loop[i].evals, rtol=0, atol=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_one_launch_batch_equals_solo(cuda, precision):
    """The instances' Davidson iterations in collective graph launches (one conditional while loop
    per solve in one graph): every instance converges to the energies of its solo solve, which
    runs the same kernels in the same order (1e-12 Eh)."""
    from forte2_gb300.batch import batched_instances, make_solver, solve_batched

    inst = batched_instances(6, seed=12)
    for x in inst:
        x["norb"] = min(x["norb"], 8)
        x["na"] = x["nb"] = x["norb"] // 2
    stats = {}
    res, _, _ = solve_batched(inst, precision, nstreams=4, one_launch=True, stats=stats)
    assert stats["batch_launches"] >= 1 and stats["batch_solves"] >= len(inst) and stats["batch_nodes"] > 0
    for i, x in enumerate(inst):
        solo = make_solver(x, precision).run()
        assert res[i].converged and solo.converged
        np.testing.assert_allclose(res[i].evals, solo.evals, rtol=0, atol=1e-12)


def test_one_launch_batch_rejects_a_shared_sigma_builder(cuda):
    import ctypes as C

    import torch

    from forte2_gb300._lib import lib
    from forte2_gb300.batch import make_solver
    from forte2_gb300.davidson import GraphPhase

    x = dict(norb=6, na=3, nb=3, multiplicity=1, nroot=1, iseed=5)
    solver = make_solver(x, "fp64", one_launch=True)
    gen = solver.run_steps()
    req = next(gen)
    while not isinstance(req, GraphPhase):
        torch.cuda.synchronize()
        req = gen.send([t.cpu().numpy() for t in req])
    arr = (C.c_void_p * 2)(req.handle.value, req.handle.value)
    b = C.c_void_p()
    assert lib().f2g_dgraph_batch_create(C.addressof(arr), 2, C.byref(b)) == 2
    assert "own sigma builder" in lib().f2g_last_error().decode()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-8)])
def test_serving_results_equal_solo(cuda, precision, tol):
    from forte2_gb300.batch import make_solver
    from forte2_gb300.serve import poisson_stream, request_precision, serve

    reqs = poisson_stream(40, rate=2000.0, seed=3, sizes=(6, 8, 10))
    # mixed_min_ndet = 0: the mixed-precision path serves these small spaces too
    stats, lat, energies = serve(reqs, precision=precision, nstreams=8, mixed_min_ndet=0)
    assert stats["requests"] == 40 and stats["max_inflight"] > 1
    assert len(lat) == 40 and all(v >= 0 for v in lat.values())
    for r in reqs[::5]:
        solo = make_solver(r.inst, request_precision(r, precision, 0)).run()
        np.testing.assert_allclose(energies[r.idx], solo.evals, rtol=0, atol=tol)


def test_serving_admission_respects_budget(cuda):
    from forte2_gb300.batch import footprint_bytes
    from forte2_gb300.serve import poisson_stream, serve

    reqs = poisson_stream(12, rate=5000.0, seed=4, sizes=(6, 8))
    one = max(footprint_bytes(r.norb, r.norb // 2, r.norb // 2, r.nroot) for r in reqs)
    stats, lat, _ = serve(reqs, hbm_budget=2 * one, nstreams=4)
    assert stats["peak_footprint_gb"] * 2**30 <= 2 * one + 1
    assert len(lat) == 12


def test_one_launch_batch_with_dense_same_spin(cuda):
    """The collective launch captures cuBLAS GEMMs inside its conditional loop bodies: mixed solves
    whose FP32 same-spin terms run as dense tensor-core GEMMs (forced through the autotuner's
    cache) converge in one-launch batches to the energies of their solo solves."""
    from forte2_gb300 import autotune
    from forte2_gb300.batch import make_solver, solve_batched

    inst = [dict(norb=n, na=n // 2, nb=n // 2, multiplicity=m, nroot=r, iseed=70 + i)
            for i, (n, m, r) in enumerate([(8, 1, 2), (10, 3, 1), (8, 3, 1), (10, 1, 2)])]
    autotune.clear_cache()
    dense = {"narrow_same_spin": 0, "persistent_opposite": 0, "tensor_cores": 1, "dense_same_spin": 1}
    for n in (8, 10):
        autotune._CACHE[(n, n // 2, n // 2, "fp32")] = {"choice": dict(dense), "ms": 0.0, "default_ms": 0.0,
                                                         "timings": []}
    try:
        stats = {}
        res, _, _ = solve_batched(inst, "mixed", nstreams=4, one_launch=True, stats=stats)
        assert stats["batch_launches"] >= 1 and stats["batch_solves"] >= len(inst)
        for i, x in enumerate(inst):
            solo = make_solver(x, "mixed").run()
            assert res[i].converged and solo.converged
            assert res[i].sigma_builder._tuned["fp32"]["dense_same_spin"] == 1
            np.testing.assert_allclose(res[i].evals, solo.evals, rtol=0, atol=1e-12)
    finally:
        autotune.clear_cache()
