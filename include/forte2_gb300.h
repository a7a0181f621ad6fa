/*
 * forte2_gb300 C ABI: determinant-CI sigma build and Davidson-Liu helpers on one GB300 GPU.
 *
 * The entry points replace the nanobind module forte2.lib.ci_helpers that the reference's
 * Python CI driver binds (forte2/api/ci_helpers_api.cc:35-200). Plain pointers and sizes only;
 * "dev" pointers are device (cudaMalloc / torch CUDA) memory, "host" pointers are host memory,
 * `stream` is a cudaStream_t (NULL = legacy default stream).
 *
 * Every function returns a status: 0 ok, 1 runtime error (Python RuntimeError), 2 invalid
 * argument (ValueError), 3 CUDA error, 4 out of device memory. The message of the last failure
 * on the calling thread is returned by f2g_last_error(). Errors use the reference's messages
 * where the reference defines one.
 *
 * Supported determinant spaces: one CAS/GAS space in C1 symmetry (all orbital irreps 0),
 * 0 <= na, nb <= norb <= 62.
 */
#ifndef FORTE2_GB300_H
#define FORTE2_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Message of the last failing call on this thread. */
const char* f2g_last_error(void);

/* Library version string. */
const char* f2g_version(void);

/* ---- CI strings: replaces CIStrings(na, nb, symmetry, orbital_symmetry, gas_min, gas_max)
 *      (forte2/ci/ci_strings.cc:26-184; binding api/ci_helpers_api.cc:55-86). Strings, 1-hole
 *      and 2-hole lists are built on the device. */
int f2g_strings_create(int na, int nb, int norb, void** out);
/* The general constructor: nspace GAS spaces of gas_size[g] orbitals each, orbsym the irreps
 * (0..7) of all orbitals space after space, gas_min[nmin] / gas_max[nmax] the electron bounds
 * per space, symmetry the state irrep. The determinants are the reference's blocks in its
 * order (ci_strings.cc:34-184, ci_occupation.cc:35-142, ci_string_class.cc:7-66,
 * ci_strings_makers.cc:13-73); the sigma, RDM and CSF calls take vectors of ndet elements in
 * that order. The RDMs, the FP32 sigma and the sigma of GAS-restricted spaces run the C1 kernels
 * on an embedding into the C1 CAS space of all orbitals (zero outside the space); the FP64 sigma
 * of a space blocked by irreps alone runs on the space's vectors (f2g_sigma_set_variant 4). */
int f2g_strings_create_general(int na, int nb, int symmetry, int nspace, const int* gas_size, const int* orbsym,
                               int nmin, const int* gas_min, int nmax, const int* gas_max, void** out);
int f2g_strings_destroy(void* strings);
/* out[10]: norb, na, nb, N0a, N0b (C1 strings), ndet (of the space), N1a, N1b, N2a, N2b */
int f2g_strings_info(void* strings, int64_t* out);
/* out[16]: trivial (the C1 space in C1 order), nirrep, GAS spaces, alpha classes, beta
 * classes, blocks, nas, nbs (strings of all classes), C1 determinants, alpha occupation
 * patterns, beta patterns, allowed pattern pairs, symmetry, ndet, 0, 0 */
int f2g_strings_blocks_info(void* strings, int64_t* out);
/* The same enumeration on the host alone (no device call), for checks: info[16] as
 * f2g_strings_blocks_info; then, where not NULL, the class strings and classes of both spins
 * (nas / nbs entries) and the block table (6 per block). */
int f2g_blocks_enumerate(int na, int nb, int symmetry, int nspace, const int* gas_size, const int* orbsym, int nmin,
                         const int* gas_min, int nmax, const int* gas_max, int64_t* info, uint64_t* amasks,
                         int32_t* aclasses, uint64_t* bmasks, int32_t* bclasses, int64_t* blocks);
/* Strings of one spin in (class, address) order (CIStrings::alpha_strings / beta_strings) and
 * their class indices. */
int f2g_strings_class_strings(void* strings, int spin, uint64_t* host_masks, int32_t* host_classes);
/* Blocks (determinant_classes, ci_string_class.cc:56-65): per block alpha class, beta class,
 * size, offset, alpha strings, beta strings. */
int f2g_strings_block_table(void* strings, int64_t* host_out);
/* Occupation patterns: alpha / beta patterns (6 ints each) and the allowed (alpha, beta) pairs
 * (gas_alpha_occupations, gas_beta_occupations, gas_occupations); NULL skips an output. */
int f2g_strings_occupations(void* strings, int32_t* host_aocc, int32_t* host_bocc, int32_t* host_pairs);
/* Occupation masks (bit p = orbital p) of one spin (0 alpha, 1 beta) in address order. */
int f2g_strings_masks(void* strings, int spin, uint64_t* host_out);
/* 1-hole list rows (class_K, K, class_I, sign, p, I), the reference's get_*_1h_list2 content
 * (ci_strings_makers.cc:163-241); host_rows = NULL returns the row count only. */
int f2g_strings_list1h(void* strings, int spin, int32_t* host_rows, int64_t* count);
/* 2-hole list rows (class_K, K, class_I, sign, p, q, I) (ci_strings_makers.cc:243-274). */
int f2g_strings_list2h(void* strings, int spin, int32_t* host_rows, int64_t* count);

/* ---- sigma builder: replaces CISigmaBuilder (forte2/ci/ci_sigma_builder.h:26-117;
 *      binding api/ci_helpers_api.cc:89-148). H is (norb, norb) row-major, V is the physicist
 *      tensor V[p][q][r][s] = <pq|rs> = (pr|qs), both host FP64. */
int f2g_sigma_create(void* strings, double E, const double* host_H, const double* host_V, int log_level,
                     void** out);
int f2g_sigma_destroy(void* sigma);
/* set_Hamiltonian (ci_sigma_builder.cc:102-185) */
int f2g_sigma_set_hamiltonian(void* sigma, double E, const double* host_H, const double* host_V);
/* set_algorithm: "kh", "knowles-handy", "hz", "harrison-zarrabian" (ci_sigma_builder.cc:49-57) */
int f2g_sigma_set_algorithm(void* sigma, const char* name);
/* get_algorithm: "Knowles-Handy" or "Harrison-Zarrabian" (ci_sigma_builder.cc:59-68) */
int f2g_sigma_get_algorithm(void* sigma, char* buf, int buflen);
/* set_memory in MB (ci_sigma_builder.cc:70-78); negative -> status 2 */
int f2g_sigma_set_memory(void* sigma, int mb);
/* 0 = FP64 (the reference's arithmetic), 1 = FP32 compute for every sigma term (mixed mode;
 * the caller refines in FP64). No reference counterpart. */
int f2g_sigma_set_precision(void* sigma, int precision);
/* Cap the thread blocks of the opposite-spin kernel (one per SM; 0 = one per alpha string, the
 * default). A capped build loops over the alpha strings and leaves the other SMs to concurrent
 * work, e.g. small latency-bound solves beside a large one. Same results. No reference counterpart. */
int f2g_sigma_set_max_blocks(void* sigma, int max_blocks);
/* FP32 precision only: compute the opposite-spin term on the tensor cores (tcgen05, operands scaled
 * by powers of two and split into two FP16 parts, three products accumulated in FP32: FP32-level
 * accuracy; the sigma row is summed in exact 64-bit fixed point, so results are bitwise
 * reproducible). *available = 1 if this space supports it (n <= 16 orbitals, na (n - na + 1) <= 72,
 * nb (n - nb + 1) <= 72, one sigma row of beta strings in shared memory); otherwise the CUDA-core
 * kernel is used. No reference counterpart. */
int f2g_sigma_set_tensor_cores(void* sigma, int on, int* available);
/* Kernel variants with identical results, for the autotuner: which = 0 opposite spin on the tensor
 * cores (FP32 only), 1 same-spin kernel with half the columns per thread, 2 opposite-spin grid of
 * one thread block per SM. which = 3 sets the polls per bounded wait of the tensor-core kernel
 * (0 = the default, about a second) and clears its error flag; a small value makes the waits give
 * up, which exercises the error path. which = 4 (default 1): the FP64 sigma of a space blocked by
 * irreps alone on its own vectors (irrep-aware opposite-spin kernel, same-spin terms block by
 * block); 0 runs the C1 kernels on the embedding (same sigma to rounding). which = 5 (default 1):
 * the tensor-core kernel's B tiles are prebuilt for every alpha string and fed by TMA; 0 builds
 * them in each thread block (the same sigma bits). which = 6: the FP32 same-spin terms as dense
 * tensor-core GEMMs (split FP16, three products; spaces of at most 4096 strings per spin, else
 * error 2; default 1 from 512 strings per spin). No reference counterpart. */
int f2g_sigma_set_variant(void* sigma, int which, int value);
/* 1 if a tensor-core build gave up waiting for its matrix operations (results invalid). */
int f2g_sigma_tc_error(void* sigma, int* out);
/* Hamiltonian(basis, sigma) for nvec vectors of length ndet stored back to back
 * (ci_sigma_builder.cc:187-218); sigma is overwritten. */
int f2g_sigma_apply(void* sigma, const double* dev_C, double* dev_sigma, int nvec, void* stream);
/* The same through host buffers: H2D copy, apply, D2H copy (end-to-end path). */
int f2g_sigma_apply_host(void* sigma, const double* host_C, double* host_sigma, int nvec);
/* One HZ term alone, overwriting dev_sigma: 0 H0, 1 H1 alpha, 2 H1 beta, 3 opposite spin,
 * 4 same-spin alpha (two-electron only), 5 same-spin beta (hz.cc:14-308). */
int f2g_sigma_term(void* sigma, int term, const double* dev_C, double* dev_sigma, void* stream);
/* avg_build_time: [total, aabb, aaaa, bbbb] seconds per build (ci_sigma_builder.h:93-102);
 * aaaa includes H0 and H1 alpha, bbbb includes H1 beta. */
int f2g_sigma_avg_build_time(void* sigma, double* host_out4);
/* Restart the build-time averages (after tuning or warm-up builds). No reference counterpart. */
int f2g_sigma_reset_build_times(void* sigma);
/* Slater-rule energy of every determinant, address order (slater_rules.cc:86-121). */
int f2g_sigma_det_energies(void* sigma, double* dev_out, void* stream);

/* ---- reduced density matrices between two determinant vectors: replaces
 *      CISigmaBuilder::compute_{a,b,sf}_1rdm (forte2/ci/ci_sigma_builder_1rdm.cc:9-84),
 *      compute_{aa,bb,ab,sf}_2rdm and compute_sf_2cumulant (ci_sigma_builder_2rdm.cc:46-282);
 *      bound as a_1rdm ... sf_2cumulant (api/ci_helpers_api.cc:110-131). */
/* Number of doubles of RDM `kind` for norb orbitals (or -1 for an unknown kind):
 * 0 a_1rdm, 1 b_1rdm, 2 sf_1rdm: norb^2, [p][q] = <L|a+_p a_q|R>;
 * 3 aa_2rdm, 4 bb_2rdm: P^2 with P = norb(norb-1)/2, [pq][rs] for p > q, r > s, pair index
 *   p(p-1)/2 + q, element <L|a+_p a+_q a_s a_r|R> of one spin;
 * 5 ab_2rdm: norb^4, [u][v][x][y] = <L|a+_u(alpha) a+_v(beta) a_y(beta) a_x(alpha)|R>;
 * 6 sf_2rdm: norb^4, ab[p][q][r][s] + ab[q][p][s][r] + the antisymmetric expansion of aa + bb;
 * 7 sf_2cumulant: norb^4, sf_2rdm[p][q][r][s] - G1[p][r] G1[q][s] + G1[p][s] G1[q][r] / 2;
 * three-body kinds (CISigmaBuilder::compute_*_3rdm, ci_sigma_builder_3rdm.cc:84-541; bound as
 * aaa_3rdm ... sf_3cumulant, api/ci_helpers_api.cc:115-139):
 * 8 aaa_3rdm, 9 bbb_3rdm: T^2 with T = norb(norb-1)(norb-2)/6, [pqr][stu] for p > q > r, s > t > u,
 *   triplet index p(p-1)(p-2)/6 + q(q-1)/2 + r;
 * 10 aab_3rdm: (P, norb, P, norb) as [pq][r][st][u] (alpha pairs p > q, s > t; beta r, u);
 * 11 abb_3rdm: (norb, P, norb, P) as [p][qr][s][tu] (alpha p, s; beta pairs q > r, t > u);
 * 12 sf_3rdm: norb^6; 13 sf_3cumulant: norb^6. The aab/abb kinds need norb <= 23. */
int64_t f2g_rdm_size(int norb, int kind);
/* RDM `kind` between the bra dev_C_left and the ket dev_C_right (device FP64, ndet each; the
 * same pointer for both selects the symmetric kernels) into dev_out (f2g_rdm_size doubles,
 * overwritten), ordered on `stream`. */
int f2g_sigma_rdm(void* sigma, int kind, const double* dev_C_left, const double* dev_C_right, double* dev_out,
                  void* stream);
/* Host-side orbital-pair list of one spin (the mixed-spin 2-RDM's work list), for inspection and
 * tests; no device call. With host_entries == NULL only counts[] is filled:
 * counts = {segments (multiple of 32), real entries, wide (0/1), padding index N0}.
 * Layout: entry j of segment g at ((g/32)*64 + j)*32 + g%32; narrow entries (32-bit)
 * left | right << 15 | negative << 30, wide (64-bit) left | right << 24 | negative << 48;
 * host_seg_pair[g] = p*norb + q. */
int f2g_rdm_pair_list(int norb, int nel, int force_wide, void* host_entries, uint16_t* host_seg_pair,
                      int64_t* host_counts4);

/* ---- two-component (relativistic) sigma builder: replaces RelCISigmaBuilder(lists, E, H, V)
 *      (forte2/ci/rel_ci_sigma_builder.cc:15-238, rel_ci_sigma_builder_harrison_zarrabian.cc;
 *      binding api/ci_helpers_api.cc:203-229). The strings must have nb == 0 (every electron an
 *      alpha spinor). H (norb x norb) and V (norb^4, physicist) are complex, stored as
 *      interleaved (re, im) doubles, as are the vectors. The default algorithm is Knowles-Handy,
 *      for which the reference applies only E (its two-component KH branch is empty); "hz" applies
 *      E + H1 + H2. */
int f2g_rel_sigma_create(void* strings, double E, const double* host_H, const double* host_V, void** out);
int f2g_rel_sigma_destroy(void* rel_sigma);
int f2g_rel_sigma_set_algorithm(void* rel_sigma, const char* name);
int f2g_rel_sigma_get_algorithm(void* rel_sigma, char* buf, int buflen);
int f2g_rel_sigma_set_memory(void* rel_sigma, int mb);
/* sigma <- H C for nvec complex vectors of ndet elements back to back (device, overwritten) */
int f2g_rel_sigma_apply(void* rel_sigma, const double* dev_C, double* dev_sigma, int nvec, void* stream);
/* form_Hdiag(dets): the complex diagonal (ndet, device) */
int f2g_rel_sigma_hdiag(void* rel_sigma, double* dev_out, void* stream);
/* slater_rules(dets, I, J) = <I|H|J> into host_out[2] */
int f2g_rel_sigma_element(void* rel_sigma, int64_t I, int64_t J, double* host_out);
/* so_1rdm ... so_3cumulant(C_left, C_right) (forte2/ci/rel_ci_sigma_builder_rdm.cc:14-404; binding
 * api/ci_helpers_api.cc:217-226): kind 0 so_1rdm (n^2), 1 so_2rdm (n^4), 2 so_2cumulant (n^4),
 * 3 so_3rdm (n^6), 4 so_3cumulant (n^6); complex interleaved, bra conjugated, row-major full
 * tensors. Vectors and output on the device; f2g_rel_rdm_size gives the complex element count
 * (-1 and the error text for a bad kind). */
int64_t f2g_rel_rdm_size(int nspinor, int kind);
int f2g_rel_sigma_rdm(void* rel_sigma, int kind, const double* dev_CL, const double* dev_CR, double* dev_out,
                      void* stream);

/* ---- spin adapter: replaces CISpinAdapter(twoS, twoMs, norb) + prepare_couplings(dets)
 *      (forte2/determinant/ci_spin_adapter.cc:55-235; binding api/ci_helpers_api.cc:190-200). */
int f2g_spin_adapter_create(void* strings, int twoS, int twoMs, void** out);
int f2g_spin_adapter_destroy(void* sa);
/* out[3]: nconf, ncsf, ncoupling (non-zero CSF-determinant overlaps) */
int f2g_spin_adapter_info(void* sa, int64_t* out);
/* csf_C_to_det_C (ci_spin_adapter.cc:84-97), nvec vectors back to back */
int f2g_csf_to_det(void* sa, const double* dev_csf, double* dev_det, int nvec, void* stream);
/* det_C_to_csf_C (ci_spin_adapter.cc:69-82) */
int f2g_det_to_csf(void* sa, const double* dev_det, double* dev_csf, int nvec, void* stream);
/* sigma in the CSF basis for nvec vectors of length ncsf (the sigma closure of ci.py:221-235 as
 * one call: csf_C_to_det_C, Hamiltonian, det_C_to_csf_C). In FP32 precision (mixed mode) the two
 * transforms also run in FP32. Scratch is kept by the spin adapter: calls on one adapter must not
 * overlap on the GPU. */
int f2g_sigma_apply_csf(void* sigma, void* sa, const double* dev_csf_in, double* dev_csf_out, int nvec,
                        void* stream);
/* form_Hdiag_csf(dets, spin_adapter, false) (ci_sigma_builder.cc:317-370) */
int f2g_hdiag_csf(void* sigma, void* sa, double* dev_out, void* stream);
/* Dense <I|H|J> over CSF indices idx[0..m) (slater_rules_csf, ci_sigma_builder.cc:278-315),
 * host_out is m x m row-major. */
int f2g_csf_matrix(void* sigma, void* sa, const int64_t* host_idx, int m, double* host_out);
/* The same with device indices and a device m x m output, ordered on stream (no host wait). */
int f2g_csf_matrix_dev(void* sigma, void* sa, const int64_t* dev_idx, int m, double* dev_out, void* stream);
/* The CSF->determinant couplings in the reference's order (bounds[ncsf+1], det index and
 * coefficient per coupling, conf_ranges[2*nconf]) for parity checks. */
int f2g_spin_adapter_dump(void* sa, int64_t* host_bounds, int64_t* host_det_idx, double* host_coeff,
                          int64_t* host_conf_ranges);

/* ---- Davidson-Liu device kernels (forte2/helpers/davidsonliu.py:184-484). Vectors are rows
 *      of length n with leading dimension ld. All FP64. `scratch` holds at least
 *      f2g_dav_scratch_size(n) doubles. */
int64_t f2g_dav_scratch_size(int64_t n);
/* out[i * nb + j] = <A_i, B_j> */
int f2g_dav_dots(const double* dev_A, int na, int64_t lda, const double* dev_B, int nb, int64_t ldb, int64_t n,
                 double* dev_out, double* dev_scratch, void* stream);
/* The same dot products for callers that cannot allocate device memory when they need them: a host
 * program whose device memory comes from its own pool (a cudaMalloc would bypass the pool and fails
 * once the pool has reserved the GPU), or one that must not add the device-wide synchronisation
 * a cudaMalloc/cudaFree can cause inside its iteration loop. No counterpart in the reference.
 * Allocates nothing and takes no scratch argument: the partial sums live in a 608 KB static
 * device array (304 blocks x 256 pairs) that every GPU loading the library holds until exit.
 * Limit: na * nb <= 256 vector pairs per call (status 2 beyond), na, nb <= 64, any n. The first
 * call on each device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture. Every call reuses the same array, so
 * calls that overlap on the GPU (other streams, other host threads) race and must be serialised.
 * The looked-up address is kept for the process: do not call this again after a cudaDeviceReset.
 * NULL operands with na * nb > 0 and negative sizes return status 2 before any device work. */
int f2g_dav_dots_noalloc(const double* dev_A, int na, int64_t lda, const double* dev_B, int nb, int64_t ldb,
                         int64_t n, double* dev_out, void* stream);
/* Y_j = beta Y_j + sum_i coef[i * ny + j] X_i (Y must not alias X) */
int f2g_dav_lincomb(const double* dev_X, int nx, int64_t ldx, const double* dev_coef, int ny, double* dev_Y,
                    int64_t ldy, double beta, int64_t n, void* stream);
/* R_r = (S alpha_r - lam_r B alpha_r) / (lam_r - hdiag) where |lam_r - hdiag| > thresh else 0;
 * norms2[r] = ||S alpha_r - lam_r B alpha_r||^2 (before preconditioning); alpha is m x nroot. */
int f2g_dav_residual(const double* dev_B, const double* dev_S, int m, int64_t ld, const double* dev_alpha,
                     const double* dev_lam, int nroot, const double* dev_hdiag, int64_t n, double thresh,
                     double* dev_R, int64_t ldr, double* dev_norms2, double* dev_scratch, void* stream);
/* Symmetric eigensolver for m <= 64: eigenvalues ascending, eigenvectors as columns (row-major). */
int f2g_dav_eigh(int m, const double* dev_G, double* dev_evals, double* dev_evecs, void* stream);
/* Gram-Schmidt with the reference's acceptance rule (davidsonliu.py:438-484) decided on the device:
 * appends the ncand rows of R, in order, to the orthonormal rows B[0, m0), then random rows until
 * m0 + added >= min_total (at most 10 tries per missing row); *dev_added receives the count. One
 * thread block does the work, so it suits vectors up to a few 10^4 elements. Needs
 * m0 + ncand <= cap, min_total <= cap, cap <= 64 (B has cap rows of leading dimension ld). */
int f2g_dav_gs_append(double* dev_B, int64_t ld, int cap, int m0, const double* dev_R, int64_t ldr, int ncand,
                      int64_t n, double discard, double ortho, int min_total, uint64_t seed, int* dev_added,
                      void* stream);

/* ---- graph-captured Davidson-Liu iterations ----------------------------------------------------
 * Replaces the host loop of DavidsonLiuSolver.solve (forte2/helpers/davidsonliu.py:184-387) driving
 * the CSF sigma closure of _CISingleStateSolver (forte2/ci/ci.py:221-235); no C++ counterpart in the
 * reference. One iteration (sigma of the new basis rows, subspace matrix, Jacobi, residuals,
 * convergence and stall tests, collapse with its orthonormality checks, projection, Gram-Schmidt)
 * is captured once into a CUDA graph of iters_per_launch iterations that reads every size and
 * decision from a device state, and ends by copying that state to pinned host memory.
 * Caller-owned device buffers: b, sigma (maxm rows, leading dimension ld), r (nroot rows, ldr),
 * tmp (2 * collapse_k rows, ldt), hdiag (n); they must outlive the handle. thresholds =
 * {preconditioner denominator, Gram-Schmidt discard, orthogonality} (1e-8, 1e-8, 1e-12 in the
 * reference). The sigma builder's precision at the first launch is the one captured. */
int f2g_dgraph_create(void* sigma, void* spin_adapter, int64_t n, int nroot, int maxm, int collapse_k,
                      int maxiter_cap, uint64_t seed, int iters_per_launch, const double* host_thresholds,
                      double* dev_b, double* dev_sigma, double* dev_r, double* dev_tmp, int64_t ld, int64_t ldr,
                      int64_t ldt, const double* dev_hdiag, void** out);
int f2g_dgraph_destroy(void* dgraph);
/* Mixed-precision phase: sigma of each new row gains D (X b) + X (D b) - X Mxd (X b) (k <= 16 rows
 * X, D of leading dimension ldx, symmetric k x k Mxd, all device). k = 0 removes it. */
int f2g_dgraph_set_correction(void* dgraph, const double* dev_X, const double* dev_D, int64_t ldx,
                              const double* dev_Mxd, int k);
/* Start a solve: basis rows [0, m) orthonormal in b, sigma current for [0, sigma_size), at most
 * nroot rows without sigma; lam_old = previous roots (nlam of them, zeros otherwise). With
 * dev_m != NULL the basis size is read on the device from *dev_m when the reset runs (m is then an
 * upper bound) and sigma_size < 0 means "sigma current for all m rows". With dev_S != NULL the
 * overlap S of the starting rows (leading dimension ldS) is checked on the device as the reference
 * checks it at the start of a solve (status 6 if it fails). */
int f2g_dgraph_reset(void* dgraph, int m, int sigma_size, const int32_t* dev_m, const double* dev_S, int ldS,
                     const double* host_lam_old, int nlam, double e_tol, double r_tol, int maxiter,
                     int stall_window, double stall_floor, void* stream);
/* Enqueue iters_per_launch iterations on stream (the first launch captures the graph). */
int f2g_dgraph_launch(void* dgraph, void* stream);
/* The state copied by the last completed launch (synchronise the stream first):
 * ints = {m, sigma_size, iterations, status, collapse, added, m_eig, 0}; status 0 running,
 * 1 converged, 2 iteration limit, 3 stalled, 4/5 basis not orthonormal before/after a collapse,
 * 6 starting basis not orthonormal (or empty);
 * doubles = {max |dE|, max |r|, the 64 subspace eigenvalues, the 64 previous roots, max |S - I| of
 * the starting basis}. */
int f2g_dgraph_state(void* dgraph, int32_t* host_ints8, double* host_doubles131);
/* Ritz vectors of the first nroot roots into rows of out (davidsonliu.py:380-387). */
int f2g_dgraph_ritz(void* dgraph, double* dev_out, int64_t ldo, void* stream);
/* Per-iteration {mean root energy, max |dE|, max |r|, basis size} of the current solve (blocking). */
int f2g_dgraph_history(void* dgraph, double* host_out, int count);
/* Many solves in ONE graph launch (batched CASCI, no reference counterpart: the reference solves
 * instances one after the other). The batch graph has one branch per dgraph: a conditional WHILE
 * node whose body is one iteration of that solve, looping until its state stops (or its
 * maxiter_cap + 2 loops), then the state copy to its host slot. Every dgraph must be reset first
 * and use its own sigma builder. f2g_dgraph_serial changes when a dgraph's captured work changes
 * (f2g_dgraph_set_correction); a batch launch rebuilds itself when one of its serials changed.
 * f2g_dgraph_batch_nodes: nodes captured into the batch. */
int f2g_dgraph_serial(void* dgraph, uint64_t* host_out);
int f2g_dgraph_batch_create(void* const* dgraphs, int count, void** out);
int f2g_dgraph_batch_destroy(void* batch);
int f2g_dgraph_batch_launch(void* batch, void* stream);
int f2g_dgraph_batch_nodes(void* batch, int* host_out);
/* set_hamiltonian ordered on a stream, with no device-wide synchronisation; buffers keep their
 * addresses for the same orbital count, so graphs captured on this builder stay valid. */
int f2g_sigma_set_hamiltonian_async(void* sigma, double E, const double* host_H, const double* host_V,
                                    void* stream);

/* ---- measurement ---------------------------------------------------------------------------- */
/* FP64 FMA issue-rate probe: blocks x threads threads each run 16 independent DFMA chains of
 * `iters` steps (32 blocks threads iters FLOP); dev_out[blocks] receives the chains' sums. The
 * roofline denominator of the FP64 sigma kernels, timed by the caller. No reference counterpart. */
int f2g_probe_dfma(int blocks, int threads, int64_t iters, double* dev_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FORTE2_GB300_H */
