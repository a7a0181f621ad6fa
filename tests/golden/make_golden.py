"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference sources are checked out, with their root in FORTE2_REFERENCE_ROOT:

    oracle/build_ref.sh "$FORTE2_REFERENCE_ROOT"
    python tests/golden/make_golden.py [--big]

Everything here comes from the reference's own code: its C++ CIStrings / CISigmaBuilder
(sigma and RDM builders) / CISpinAdapter compiled unmodified by oracle/build_ref.sh, and its helpers/davidsonliu.py
driven exactly as forte2/ci/ci.py:245-303 drives it (CSF basis, Hdiag from form_Hdiag_csf,
guess vectors from ci.py:411-452, sigma closure from ci.py:221-235). Integrals are the seeded
synthetic recipe of forte2_gb300.synthetic. The fixtures are small .npz files; large cases are
stored as checksums (norms, dot products with seeded vectors, sampled entries, SHA-256 of the
integer lists) so they can be checked at full size without committing the full vectors.
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from forte2_gb300.synthetic import make_integrals, random_ci_vector  # noqa: E402
from oracle import reference as ref  # noqa: E402
from oracle.ref_davidson import load as load_davidson  # noqa: E402

# (na, nb, norb) for the string/list fixtures, including empty and one-electron edge cases.
LIST_CASES = [(0, 0, 3), (1, 0, 3), (0, 1, 3), (1, 1, 1), (1, 1, 2), (2, 2, 4), (3, 3, 6),
              (2, 4, 7), (4, 4, 8), (3, 5, 9), (5, 5, 10), (6, 6, 12), (7, 7, 14)]
LIST_HASH_CASES = [(8, 8, 16)]

# (na, nb, norb, integral seed, vector seed) for sigma fixtures.
SIGMA_CASES = [(1, 1, 2, 11, 101), (2, 2, 4, 12, 102), (3, 3, 6, 13, 103), (2, 3, 6, 14, 104),
               (3, 1, 6, 15, 105), (1, 4, 6, 16, 106), (4, 0, 6, 17, 107), (0, 3, 5, 18, 108),
               (4, 4, 8, 19, 109), (5, 5, 10, 1000, 110), (4, 5, 9, 21, 111)]
SIGMA_CHECKSUM_CASES = [(6, 6, 12, 22, 112), (7, 7, 14, 2000, 113)]
SIGMA_CHECKSUM_BIG = [(8, 8, 16, 3000, 114)]

# (na, nb, norb, bra seed, ket seed) for the reduced-density-matrix fixtures: every RDM kind of
# the reference between two different vectors and of one vector with itself.
RDM_CASES = [(1, 1, 1, 201, 202), (1, 1, 2, 203, 204), (2, 2, 4, 205, 206), (3, 3, 6, 207, 208),
             (2, 3, 6, 209, 210), (3, 1, 6, 211, 212), (1, 4, 6, 213, 214), (4, 0, 6, 215, 216),
             (0, 3, 5, 217, 218), (3, 2, 7, 219, 220), (4, 4, 8, 221, 222)]

# (na, nb, norb, multiplicity, twice_ms, nroot, integral seed, e_tol, maxiter). The CAS(10,10)
# four-root case does not converge within the reference's default 100 iterations on these
# integrals, so it is also run with a larger iteration cap.
DAVIDSON_CASES = [(2, 2, 4, 1, 0, 2, 31, 1e-12, 100), (3, 3, 6, 1, 0, 3, 32, 1e-12, 100),
                  (3, 3, 6, 3, 0, 2, 33, 1e-12, 100), (4, 3, 7, 2, 1, 2, 34, 1e-12, 100),
                  (4, 4, 8, 1, 0, 4, 35, 1e-12, 100), (4, 4, 8, 3, 0, 3, 36, 1e-12, 100),
                  (5, 5, 10, 1, 0, 4, 1000, 1e-10, 100), (5, 5, 10, 1, 0, 4, 1000, 1e-10, 1000)]


def list_rows(s: ref.RefCIStrings, spin: int):
    return s.list_1h(spin), s.list_2h(spin)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gen_lists(out):
    data = {}
    meta = {}
    for na, nb, n in LIST_CASES:
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        key = f"{na}_{nb}_{n}"
        for spin, tag in ((0, "a"), (1, "b")):
            masks, classes = s.strings(spin)
            l1, l2 = list_rows(s, spin)
            l1k = s.list_1h(spin, keyed=True)
            assert np.array_equal(l1, l1k), "1h list2 and keyed 1h list disagree"
            data[f"{key}_{tag}_strings"] = masks
            data[f"{key}_{tag}_1h"] = l1
            data[f"{key}_{tag}_2h"] = l2
        meta[key] = dict(nas=s.nas, nbs=s.nbs, ndet=s.ndet)
    for na, nb, n in LIST_HASH_CASES:
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        key = f"{na}_{nb}_{n}"
        for spin, tag in ((0, "a"), (1, "b")):
            masks, _ = s.strings(spin)
            l1, l2 = list_rows(s, spin)
            meta[f"{key}_{tag}"] = dict(strings_sha=sha(masks), l1_sha=sha(l1), l2_sha=sha(l2),
                                        n_strings=len(masks), n_1h=len(l1), n_2h=len(l2))
        meta[key] = dict(nas=s.nas, nbs=s.nbs, ndet=s.ndet)
    np.savez_compressed(os.path.join(out, "lists.npz"), **data)
    with open(os.path.join(out, "lists_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


def spin_of(na, nb):
    return abs(na - nb)


def gen_sigma(out):
    data = {}
    for na, nb, n, iseed, cseed in SIGMA_CASES:
        ints = make_integrals(n, iseed)
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
        sb.set_algorithm("hz")
        c = random_ci_vector(s.ndet, cseed)
        sig = np.zeros(s.ndet)
        sb.Hamiltonian(c, sig)
        key = f"{na}_{nb}_{n}"
        small = s.ndet <= 5000
        # C is regenerated from its seed by random_ci_vector; its hash guards the recipe.
        data[f"{key}_C_sha"] = np.frombuffer(sha(c).encode(), dtype=np.uint8)
        data[f"{key}_sigma"] = sig
        for t in sb.TERMS if small else ("aabb", "aaaa", "bbbb"):
            data[f"{key}_term_{t}"] = sb.term(t, c)
        if small:
            sbk = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
            sbk.set_algorithm("kh")
            sk = np.zeros(s.ndet)
            sbk.Hamiltonian(c, sk)
            data[f"{key}_sigma_kh"] = sk
        if small:
            data[f"{key}_det_energies"] = sb.det_energies()
        data[f"{key}_V_sha"] = np.frombuffer(sha(ints.V).encode(), dtype=np.uint8)
        data[f"{key}_seeds"] = np.array([iseed, cseed])
        # spin adaptation: lowest multiplicity compatible with Ms, and the next one
        twice_ms = na - nb
        for twoS in (abs(twice_ms), abs(twice_ms) + 2):
            if twoS > na + nb or (na + nb) == 0:
                continue
            sa = ref.RefSpinAdapter(twoS, twice_ms, n)
            sa.prepare_couplings(s)
            if sa.ncsf == 0:
                continue
            tag = f"{key}_S{twoS}"
            if not small and twoS != abs(twice_ms):
                continue
            if small:
                bounds, det_idx, coeff, ranges = sa.couplings()
                data[f"{tag}_bounds"] = bounds
                data[f"{tag}_det_idx"] = det_idx
                data[f"{tag}_coeff"] = coeff
                data[f"{tag}_conf_ranges"] = ranges
            data[f"{tag}_info"] = np.array([sa.nconf, sa.ncsf, sa.ncoupling])
            data[f"{tag}_hdiag"] = sb.form_Hdiag_csf(sa)
            csf = random_ci_vector(sa.ncsf, cseed + 7)
            data[f"{tag}_csf_to_det"] = sa.csf_C_to_det_C(csf)
            data[f"{tag}_det_to_csf"] = sa.det_C_to_csf_C(sig)
            m = min(sa.ncsf, 12)
            data[f"{tag}_slater_csf"] = np.array(
                [[sb.slater_rules_csf(sa, i, j) for j in range(m)] for i in range(m)])
    np.savez_compressed(os.path.join(out, "sigma.npz"), **data)


def gen_rdm(out):
    data = {}
    for na, nb, n, sl, sr in RDM_CASES:
        ints = make_integrals(n, sl)
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
        cl = random_ci_vector(s.ndet, sl)
        cr = random_ci_vector(s.ndet, sr)
        key = f"{na}_{nb}_{n}"
        data[f"{key}_seeds"] = np.array([sl, sr])
        data[f"{key}_CL_sha"] = np.frombuffer(sha(cl).encode(), dtype=np.uint8)
        data[f"{key}_CR_sha"] = np.frombuffer(sha(cr).encode(), dtype=np.uint8)
        for kind in sb.RDM_KINDS:
            data[f"{key}_{kind}_LR"] = sb.rdm(kind, cl, cr)
            data[f"{key}_{kind}_LL"] = sb.rdm(kind, cl, cl)
    np.savez_compressed(os.path.join(out, "rdm.npz"), **data)


RDM3_KINDS = ("aaa_3rdm", "bbb_3rdm", "aab_3rdm", "abb_3rdm", "sf_3rdm", "sf_3cumulant")


def rdm_checksum(a, seed):
    """Compact pin of a large array: its norm, its dot product with a seeded normal vector and
    64 entries at seeded positions."""
    a = np.asarray(a).reshape(-1)
    if a.size == 0:
        return dict(size=0)
    rng = np.random.default_rng(seed)
    w = rng.normal(size=a.size)
    idx = np.sort(rng.choice(a.size, size=min(64, a.size), replace=False))
    return dict(size=int(a.size), norm=float(np.linalg.norm(a)), dot_w=float(a @ w), idx=idx.tolist(),
                vals=a[idx].tolist())


def gen_rdm3(out):
    """The reference's 3-RDMs (ci_sigma_builder_3rdm.cc) on the RDM_CASES vectors: checksums for
    every case, full arrays for the spaces of at most 4 orbitals."""
    data, meta = {}, {}
    for na, nb, n, sl, sr in RDM_CASES:
        ints = make_integrals(n, sl)
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
        cl = random_ci_vector(s.ndet, sl)
        cr = random_ci_vector(s.ndet, sr)
        key = f"{na}_{nb}_{n}"
        for j, kind in enumerate(RDM3_KINDS):
            for tag, b in (("LR", cr), ("LL", cl)):
                a = sb.rdm(kind, cl, b)
                meta[f"{key}_{kind}_{tag}"] = rdm_checksum(a, 7000 + 10 * j + (tag == "LL"))
                if n <= 4:
                    data[f"{key}_{kind}_{tag}"] = a
    np.savez_compressed(os.path.join(out, "rdm3.npz"), **data)
    with open(os.path.join(out, "rdm3_checksums.json"), "w") as f:
        json.dump(meta, f)


def checksums(sig, ndet, seed):
    rng = np.random.default_rng(seed)
    w = rng.normal(size=ndet)
    idx = np.sort(rng.choice(ndet, size=min(4096, ndet), replace=False))
    return dict(norm=float(np.linalg.norm(sig)), dot_w=float(sig @ w), idx=idx.tolist(),
                vals=sig[idx].tolist(), sum=float(sig.sum()))


def gen_sigma_checksums(out, cases, fname):
    meta = {}
    for na, nb, n, iseed, cseed in cases:
        t0 = time.time()
        ints = make_integrals(n, iseed)
        s = ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
        sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
        sb.set_algorithm("hz")
        c = random_ci_vector(s.ndet, cseed)
        sig = np.zeros(s.ndet)
        sb.Hamiltonian(c, sig)
        meta[f"{na}_{nb}_{n}"] = dict(iseed=iseed, cseed=cseed, ndet=s.ndet, V_sha=sha(ints.V),
                                      seconds=time.time() - t0, **checksums(sig, s.ndet, cseed + 1))
        print(f"sigma checksum {na},{nb},{n}: {time.time() - t0:.1f}s", flush=True)
    with open(os.path.join(out, fname), "w") as f:
        json.dump(meta, f)


def reference_casci(na, nb, n, mult, twice_ms, nroot, iseed, e_tol, DavidsonLiuSolver, Params,
                    maxiter=100, ints=None, solver=None, return_solver=False, space=None):
    """Drive the reference Davidson exactly as forte2/ci/ci.py:_do_iterative_ci does. With `solver`
    (a DavidsonLiuSolver that has already solved), it continues from that solver's vectors with the
    new integrals, as the reference's MCSCF loop does (ci.py:266-290, mc_optimizer.py:297-328)."""
    ints = make_integrals(n, iseed) if ints is None else ints
    # space: (symmetry, orbital_symmetry, gas_min, gas_max) of a blocked space, else C1 CAS
    s = ref.RefCIStrings(na, nb, *space) if space else ref.RefCIStrings(na, nb, 0, [[0] * n], [], [])
    sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
    sb.set_algorithm("hz")
    sa = ref.RefSpinAdapter(mult - 1, twice_ms, n)
    sa.prepare_couplings(s)
    hdiag = sb.form_Hdiag_csf(sa)
    params = Params(e_tol=e_tol, maxiter=maxiter)
    warm = solver is not None
    if not warm:
        solver = DavidsonLiuSolver(size=sa.ncsf, nroot=nroot, davidson_liu_params=params, log_level=0)
    solver.add_h_diag(hdiag)
    # guess vectors (ci.py:411-452)
    nguess = min(params.guess_per_root * nroot, sa.ncsf)
    nguess_dets = min(params.ndets_per_guess * nguess, sa.ncsf)
    indices = np.argsort(hdiag)[:nguess_dets]
    Hg = np.zeros((nguess_dets, nguess_dets))
    for i, I in enumerate(indices):
        for j, J in enumerate(indices):
            if i >= j:
                v = sb.slater_rules_csf(sa, I, J)
                Hg[i, j] = v
                Hg[j, i] = v
    _, vecs = np.linalg.eigh(Hg)
    guess = np.zeros((sa.ncsf, nguess))
    for i in range(nguess):
        for j, d in enumerate(indices):
            guess[d, i] = vecs[j, i]
    if not warm:
        solver.add_guesses(guess)

    def sigma_builder(B, S):
        for i in range(B.shape[1]):
            bd = sa.csf_C_to_det_C(np.ascontiguousarray(B[:, i]))
            sd = np.zeros(s.ndet)
            sb.Hamiltonian(bd, sd)
            S[:, i] = sa.det_C_to_csf_C(sd)

    solver.add_sigma_builder(sigma_builder)
    t0 = time.time()
    evals, evecs = solver.solve()
    seconds = time.time() - t0
    # independent cross-check: Lanczos on the same reference sigma in the CSF basis
    from scipy.sparse.linalg import LinearOperator, eigsh

    def mv(x):
        x = np.asarray(x, dtype=np.float64).reshape(-1)
        sd = np.zeros(s.ndet)
        sb.Hamiltonian(sa.csf_C_to_det_C(x), sd)
        return sa.det_C_to_csf_C(sd)

    if sa.ncsf <= 400:
        Hd = np.column_stack([mv(e) for e in np.eye(sa.ncsf)])
        lanczos = np.linalg.eigvalsh(0.5 * (Hd + Hd.T))[:nroot]
    else:
        op = LinearOperator((sa.ncsf, sa.ncsf), matvec=mv, dtype=np.float64)
        lanczos = np.sort(eigsh(op, k=nroot, which="SA", tol=1e-14, ncv=max(4 * nroot, 40))[0])
    out = dict(evals=[float(x) for x in evals], converged=bool(solver.converged),
               iterations=int(solver.iter), ncsf=sa.ncsf, ndet=s.ndet, seconds=seconds,
               hdiag_min=float(hdiag.min()), nguess_dets=int(nguess_dets), maxiter=maxiter,
               lanczos=[float(x) for x in lanczos],
               max_dev_vs_lanczos=float(np.max(np.abs(np.sort(evals) - lanczos))))
    return (out, solver) if return_solver else out


def gen_davidson(out, ref_root):
    DL, Params = load_davidson(ref_root)
    meta = {}
    for case in DAVIDSON_CASES:
        na, nb, n, mult, tms, nroot, iseed, e_tol, maxiter = case
        r = reference_casci(na, nb, n, mult, tms, nroot, iseed, e_tol, DL, Params, maxiter)
        r.update(dict(na=na, nb=nb, norb=n, multiplicity=mult, twice_ms=tms, nroot=nroot,
                      iseed=iseed, e_tol=e_tol))
        meta[f"{na}_{nb}_{n}_m{mult}_r{nroot}_it{maxiter}"] = r
        print("davidson", case, r["evals"], r["iterations"], flush=True)
    with open(os.path.join(out, "davidson.json"), "w") as f:
        json.dump(meta, f, indent=1)


# Spaces with point-group irreps and GAS restrictions (the reference's determinant blocks):
# (na, nb, symmetry, orbital_symmetry, gas_min, gas_max, integral seed, vector seed, symmetric
# integrals). The last one has no determinants.
BLOCK_CASES = [(3, 3, 1, [[0, 0, 1, 2, 3, 0]], [], [], 61, 601, False),
               (3, 3, 0, [[0, 0, 0], [0, 0, 0]], [4], [6], 62, 602, False),
               (2, 2, 0, [[0, 0], [0, 0]], [0, 0], [4, 4], 63, 603, False),
               (4, 3, 3, [[0, 1, 2, 3, 0, 1, 2, 3]], [], [], 64, 604, True),
               (3, 3, 0, [[0, 1, 0], [1, 0, 1], [0, 0]], [2, 2, 0], [6, 4, 2], 65, 605, True),
               (4, 4, 2, [[0, 2, 1], [3, 0, 1, 2], [0]], [3, 1], [6, 6, 1], 66, 606, False),
               (3, 3, 5, [[0, 1, 2, 3, 4, 5, 6, 7]], [], [], 67, 607, True),
               (4, 4, 0, [[0, 0], [0, 0, 0], [0, 0, 0]], [2, 2, 0], [4, 6, 2], 68, 608, False),
               (1, 2, 0, [[1, 1, 0]], [], [], 70, 610, False),
               (5, 4, 1, [[0, 1, 0, 1, 0], [1, 0, 1, 0, 1]], [3], [8], 71, 611, True),
               (2, 3, 0, [[1, 1, 1, 1]], [], [], 69, 609, False)]

# CASCI in blocked spaces: (na, nb, symmetry, orbital_symmetry, gas_min, gas_max, multiplicity,
# nroot, integral seed, symmetric integrals)
BLOCK_CASCI_CASES = [(4, 4, 0, [[0, 1, 2, 3, 0, 1, 2, 3]], [], [], 1, 2, 81, True),
                     (4, 4, 2, [[0, 1, 2, 3, 0, 1, 2, 3]], [], [], 3, 1, 82, True),
                     (3, 3, 0, [[0, 0, 0], [0, 0, 0]], [4], [6], 1, 2, 83, False),
                     (5, 5, 0, [[0, 0, 0, 0, 0], [0, 0, 0, 0, 0]], [6, 0], [10, 4], 1, 3, 84, False),
                     (5, 4, 1, [[0, 1, 0, 1, 0], [1, 0, 1, 0, 1]], [3], [8], 2, 2, 85, True)]


def block_ints(n, iseed, orbsym, symmetric):
    from forte2_gb300.synthetic import symmetrize_integrals

    ints = make_integrals(n, iseed)
    return symmetrize_integrals(ints, [x for g in orbsym for x in g]) if symmetric else ints


def gen_blocks(out, ref_root):
    """Blocked spaces: the reference's class strings, blocks, sigma of a seeded vector,
    determinant energies, CSF couplings and CSF diagonal; CASCI energies from the reference's
    Davidson on its compiled blocked sigma."""
    data = {}
    meta = {"cases": [], "casci": {}}
    for k, (na, nb, sym, orbsym, gmin, gmax, iseed, cseed, symm) in enumerate(BLOCK_CASES):
        n = sum(len(g) for g in orbsym)
        s = ref.RefCIStrings(na, nb, sym, orbsym, gmin, gmax)
        key = f"b{k}"
        meta["cases"].append(dict(key=key, na=na, nb=nb, symmetry=sym, orbital_symmetry=orbsym, gas_min=gmin,
                                  gas_max=gmax, iseed=iseed, cseed=cseed, symmetric=symm, ndet=s.ndet,
                                  nas=s.nas, nbs=s.nbs, nirrep=s.nirrep))
        for spin, tag in ((0, "a"), (1, "b")):
            m, c = s.strings(spin)
            data[f"{key}_{tag}_strings"] = m
            data[f"{key}_{tag}_classes"] = c
        data[f"{key}_blocks"] = s.blocks()
        data[f"{key}_dets"] = s.determinants()
        if s.ndet == 0:
            continue
        ints = block_ints(n, iseed, orbsym, symm)
        sb = ref.RefSigmaBuilder(s, ints.E, ints.H, ints.V)
        sb.set_algorithm("hz")
        c = random_ci_vector(s.ndet, cseed)
        sig = np.zeros(s.ndet)
        sb.Hamiltonian(c, sig)
        data[f"{key}_sigma"] = sig
        data[f"{key}_det_energies"] = sb.det_energies()
        twice_ms = na - nb
        for twoS in (abs(twice_ms), abs(twice_ms) + 2):
            sa = ref.RefSpinAdapter(twoS, twice_ms, n)
            sa.prepare_couplings(s)
            if sa.ncsf == 0:
                continue
            bounds, det_idx, coeff, ranges = sa.couplings()
            tag = f"{key}_S{twoS}"
            data[f"{tag}_bounds"] = bounds
            data[f"{tag}_det_idx"] = det_idx
            data[f"{tag}_coeff"] = coeff
            data[f"{tag}_ranges"] = ranges
            data[f"{tag}_hdiag"] = sb.form_Hdiag_csf(sa)
        print("blocks", key, s.ndet, flush=True)
    np.savez_compressed(os.path.join(out, "blocks.npz"), **data)
    DL, Params = load_davidson(ref_root)
    for k, (na, nb, sym, orbsym, gmin, gmax, mult, nroot, iseed, symm) in enumerate(BLOCK_CASCI_CASES):
        n = sum(len(g) for g in orbsym)
        ints = block_ints(n, iseed, orbsym, symm)
        r = reference_casci(na, nb, n, mult, na - nb, nroot, iseed, 1e-12, DL, Params, 400, ints=ints,
                            space=(sym, orbsym, gmin, gmax))
        r.update(dict(na=na, nb=nb, symmetry=sym, orbital_symmetry=orbsym, gas_min=gmin, gas_max=gmax,
                      multiplicity=mult, nroot=nroot, iseed=iseed, symmetric=symm))
        meta["casci"][f"c{k}"] = r
        print("blocks casci", k, r["evals"], r["iterations"], r["max_dev_vs_lanczos"], flush=True)
    with open(os.path.join(out, "blocks.json"), "w") as f:
        json.dump(meta, f, indent=1)


# Two-component (spinor) spaces: (spinors, electrons, orbital_symmetry or None, integral seed,
# vector seed). nb = 0: every electron is an alpha spinor.
REL_CASES = [(4, 1, None, 91, 901), (6, 0, None, 92, 902), (8, 3, None, 93, 903), (10, 4, None, 94, 904),
             (12, 5, None, 95, 905), (14, 6, None, 96, 906), (8, 4, [[0, 1, 0, 1, 0, 1, 0, 1]], 97, 907)]


def gen_rel(out):
    """The reference's RelCISigmaBuilder: sigma of a seeded complex vector (hz), the kh result,
    form_Hdiag, a few slater_rules elements; for the small spaces the lowest eigenvalues of the
    dense Hamiltonian built from its sigma."""
    from forte2_gb300.synthetic import make_spinor_integrals, random_complex_vector

    data = {}
    meta = []
    for k, (n, ne, orbsym, iseed, cseed) in enumerate(REL_CASES):
        E, H, V = make_spinor_integrals(n, iseed)
        space = (1 if orbsym else 0, orbsym, [], []) if orbsym else (0, [[0] * n], [], [])
        s = ref.RefCIStrings(ne, 0, *space)
        sb = ref.RefRelSigmaBuilder(s, E, H, V)
        key = f"r{k}"
        c = random_complex_vector(s.ndet, cseed)
        sig_kh = np.zeros(s.ndet, dtype=np.complex128)
        sb.Hamiltonian(c, sig_kh)  # the default algorithm
        sb.set_algorithm("hz")
        sig = np.zeros(s.ndet, dtype=np.complex128)
        sb.Hamiltonian(c, sig)
        data[f"{key}_sigma"] = sig
        data[f"{key}_sigma_kh"] = sig_kh
        data[f"{key}_hdiag"] = sb.form_Hdiag()
        rng = np.random.default_rng(cseed)
        pairs = rng.integers(0, max(1, s.ndet), size=(12, 2))
        data[f"{key}_pairs"] = pairs
        data[f"{key}_elements"] = np.array([sb.slater_rules(i, j) for i, j in pairs], dtype=np.complex128)
        entry = dict(key=key, nspinor=n, nel=ne, orbital_symmetry=orbsym, iseed=iseed, cseed=cseed, ndet=s.ndet)
        if s.ndet <= 800:
            Hd = np.zeros((s.ndet, s.ndet), dtype=np.complex128)
            for i in range(s.ndet):
                e = np.zeros(s.ndet, dtype=np.complex128)
                e[i] = 1.0
                o = np.zeros(s.ndet, dtype=np.complex128)
                sb.Hamiltonian(e, o)
                Hd[:, i] = o
            entry["hermitian_dev"] = float(np.abs(Hd - Hd.conj().T).max())
            entry["evals"] = [float(x) for x in np.linalg.eigvalsh(0.5 * (Hd + Hd.conj().T))[:4]]
        meta.append(entry)
        print("rel", key, s.ndet, flush=True)
    np.savez_compressed(os.path.join(out, "rel.npz"), **data)
    with open(os.path.join(out, "rel.json"), "w") as f:
        json.dump(meta, f, indent=1)


# spin-orbital RDM cases: (nspinor, nel, orbital symmetry or None, integral seed, vector seed)
REL_RDM_CASES = [(6, 3, None, 98, 908), (8, 3, None, 93, 903), (8, 4, [[0, 1, 0, 1, 0, 1, 0, 1]], 97, 907),
                 (10, 4, None, 94, 904), (4, 1, None, 91, 901), (6, 0, None, 92, 902), (5, 5, None, 99, 909)]
REL_RDM_SAMPLE = 4096  # sampled entries of a three-body tensor above 6 spinors


def gen_rel_rdm(out):
    """The reference's so_1rdm ... so_3cumulant between two seeded complex vectors (transition
    RDMs, bra conjugated) and so_1rdm / so_2rdm of one vector with itself. Three-body tensors are
    stored whole up to 6 spinors; above that, REL_RDM_SAMPLE seeded flat entries and the sum of
    squared moduli of the whole tensor."""
    from forte2_gb300.synthetic import make_spinor_integrals, random_complex_vector

    data = {}
    meta = []
    for k, (n, ne, orbsym, iseed, cseed) in enumerate(REL_RDM_CASES):
        E, H, V = make_spinor_integrals(n, iseed)
        space = (1, orbsym, [], []) if orbsym else (0, [[0] * n], [], [])
        s = ref.RefCIStrings(ne, 0, *space)
        sb = ref.RefRelSigmaBuilder(s, E, H, V)
        key = f"q{k}"
        cl = random_complex_vector(s.ndet, cseed)
        cr = random_complex_vector(s.ndet, cseed + 1)
        entry = dict(key=key, nspinor=n, nel=ne, orbital_symmetry=orbsym, iseed=iseed, cseed=cseed, ndet=s.ndet)
        for kind in ref.RefRelSigmaBuilder.RDM_KINDS:
            x = sb.rdm(kind, cl, cr)
            if kind.startswith("so_3") and n > 6:
                idx = np.random.default_rng(cseed + 7).integers(0, x.size, size=REL_RDM_SAMPLE)
                data[f"{key}_{kind}_idx"] = idx
                data[f"{key}_{kind}"] = x.reshape(-1)[idx]
                entry[f"{kind}_sumsq"] = float(np.sum(np.abs(x) ** 2))
            else:
                data[f"{key}_{kind}"] = x
        data[f"{key}_so_1rdm_diag"] = sb.rdm("so_1rdm", cl, cl)
        data[f"{key}_so_2rdm_diag"] = sb.rdm("so_2rdm", cl, cl)
        meta.append(entry)
        print("rel rdm", key, s.ndet, flush=True)
    np.savez_compressed(os.path.join(out, "rel_rdm.npz"), **data)
    with open(os.path.join(out, "rel_rdm.json"), "w") as f:
        json.dump(meta, f, indent=1)


# MCSCF-style sequence: (na, nb, norb, multiplicity, nroot, integral seed, rotation seeds, theta, e_tol)
MCSCF_CASES = [(4, 4, 8, 1, 2, 4100, (4111, 4122), 0.05, 1e-10),
               (5, 5, 10, 1, 1, 4200, (4211, 4222), 0.03, 1e-10),
               (4, 4, 8, 3, 1, 4300, (4311, 4322), 0.05, 1e-10)]


def gen_mcscf(out, ref_root):
    """Energies of successive CI solves with rotated integrals, one reference Davidson solver
    warm-started from solve to solve, as the reference's orbital optimiser drives its CI solver
    (mcopt/mc_optimizer.py:297-328: set_ints then run, ci.py:266-290 keeps the eigensolver)."""
    from forte2_gb300.synthetic import rotate_integrals

    DL, Params = load_davidson(ref_root)
    meta = {}
    for na, nb, n, mult, nroot, iseed, rseeds, theta, e_tol in MCSCF_CASES:
        ints = make_integrals(n, iseed)
        solver = None
        steps = []
        for k in range(len(rseeds) + 1):
            if k > 0:
                ints = rotate_integrals(ints, rseeds[k - 1], theta)
            r, solver = reference_casci(na, nb, n, mult, 0, nroot, iseed, e_tol, DL, Params, 400, ints=ints,
                                        solver=solver, return_solver=True)
            steps.append(dict(evals=r["evals"], iterations=r["iterations"], converged=r["converged"],
                              lanczos=r["lanczos"], max_dev_vs_lanczos=r["max_dev_vs_lanczos"],
                              H_sha=sha(ints.H)))
            print("mcscf", (na, nb, n, mult, nroot), k, r["evals"], r["iterations"], flush=True)
        meta[f"{na}_{nb}_{n}_m{mult}_r{nroot}"] = dict(na=na, nb=nb, norb=n, multiplicity=mult, nroot=nroot,
                                                      iseed=iseed, rotation_seeds=list(rseeds), theta=theta,
                                                      e_tol=e_tol, steps=steps)
    with open(os.path.join(out, "mcscf.json"), "w") as f:
        json.dump(meta, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FORTE2_REFERENCE_ROOT"),
                    required=os.environ.get("FORTE2_REFERENCE_ROOT") is None,
                    help="root of the forte2 checkout (or set FORTE2_REFERENCE_ROOT)")
    ap.add_argument("--big", action="store_true", help="also the CAS(16,16) sigma checksum")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    ref.open_blas(threads=os.cpu_count())
    steps = {"lists": lambda: gen_lists(HERE), "sigma": lambda: gen_sigma(HERE),
             "checksums": lambda: gen_sigma_checksums(HERE, SIGMA_CHECKSUM_CASES, "sigma_checksums.json"),
             "davidson": lambda: gen_davidson(HERE, a.reference), "rdm": lambda: gen_rdm(HERE),
             "mcscf": lambda: gen_mcscf(HERE, a.reference), "blocks": lambda: gen_blocks(HERE, a.reference),
             "rel": lambda: gen_rel(HERE),
             "rel_rdm": lambda: gen_rel_rdm(HERE),
             "rdm3": lambda: gen_rdm3(HERE)}
    if a.big:
        steps["big"] = lambda: gen_sigma_checksums(HERE, SIGMA_CHECKSUM_BIG, "sigma_checksums_16.json")
    for name, f in steps.items():
        if a.only and name not in a.only.split(","):
            continue
        t0 = time.time()
        f()
        print(f"{name}: {time.time() - t0:.1f}s", flush=True)


if __name__ == "__main__":
    main()
