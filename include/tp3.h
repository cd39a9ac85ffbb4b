/*
 * tp3.h -- C ABI of the GB300 c3 + Bayes scorer (libtp3.so).
 *
 * One hot path of ThreePhotons.jl: spherical-harmonic intensity coefficients of
 * K shells up to order L  ->  model three-photon correlation c3(k1,k2,k3,alpha,beta)
 *  ->  "Bayes" log-likelihood against a triplet histogram.
 *
 * Reference interfaces replaced (file:line inside ThreePhotons.jl):
 *   src/cuda.jl:10-22        CUDA_init                      -> tp3_ctx_create (device side)
 *   src/cuda.jl:45-69        CUDA_store_basis / CUDA_calculate_basis,
 *   src/correlations.jl:87-153 calculate_basis              -> tp3_ctx_create (tables)
 *   src/cuda.jl:74-108       FullCorrelation_parallized(::BasisTypeCuda) -> tp3_c3
 *   src/correlations.jl:179-193 FullCorrelation_parallized(::BasisType)  -> tp3_c3
 *   src/correlations.jl:201-226 energy(..., "Bayes")         -> tp3_energy, tp3_energy_batch
 *   src/cuda_kernel.cu:18    calculate_coefficient_matrix (PTX entry bound by
 *                            cudacall at src/cuda.jl:82-86) + cublasSgemm_v2 at
 *                            src/cuda.jl:88                  -> internal kernels of tp3_c3/tp3_energy
 *   src/datagen.jl:432-475   loadHistograms' c3 contract     -> tp3_set_histogram
 *   src/determination.jl:281-338, 491-515 rotate_all_at_once / evaluate_step
 *                                                            -> tp3_chains_* (device-resident chains)
 *
 * Conventions
 *   - Every call returns an int status (TP3_OK = 0).  There is no CPU fallback:
 *     without a usable GPU the calls fail with TP3_ERR_NO_DEVICE / TP3_ERR_CUDA.
 *   - Host pointers are only read (or written, for outputs) during the call.
 *   - Coefficients: interleaved (re, im) doubles, shell-major: shell k (0-based)
 *     occupies doubles [2*LMAX^2*k, 2*LMAX^2*(k+1)), entry (l, m) at the
 *     reference's seanindex(l, m, LMAX) - 1 (src/spherical_harmonics.jl:163-170).
 *   - c3 output: 2N^2 x klength column-major float (the reference's raw
 *     `return_raw=true` layout, src/cuda.jl:91): grid row g = a + N*b, column ki
 *     enumerating k1 >= k2 >= k3 with k1 outermost (src/correlations.jl:72-81).
 *   - Histogram: N x 2N x K3 x K3 x K3 column-major doubles (Julia's C3 array,
 *     element (a, b, k3, k2, k1)), K3 >= K.
 *   - One context = one CUDA stream; calls on a context must be serialised by the
 *     caller.  Contexts are independent.
 */
#ifndef TP3_H
#define TP3_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TP3_OK 0
#define TP3_ERR_ARG 1            /* bad argument or shape */
#define TP3_ERR_TABLE 2          /* table construction failed an invariant */
#define TP3_ERR_CUDA 3           /* CUDA runtime error */
#define TP3_ERR_NO_DEVICE 4      /* no usable CUDA device */
#define TP3_ERR_NO_HISTOGRAM 5   /* energy requested before tp3_set_histogram */
#define TP3_ERR_BAD_HISTOGRAM 6  /* NaN/Inf value or a slab with zero L1 norm */
#define TP3_ERR_TIMEOUT 7        /* a bounded device wait ran out */
#define TP3_ERR_UNSUPPORTED 8    /* mode not available for this (L, K, N, lambda) */
#define TP3_ERR_ALLOC 9          /* device or host allocation failed */
#define TP3_ERR_BOUNDS 10        /* a TP3_DEBUG build's device index check failed (access skipped) */

/* Evaluation modes (tp3_set_mode). */
#define TP3_MODE_PLAIN_FP32 0    /* direct coupling + FP32 SIMT angular contraction, full grid */
#define TP3_MODE_TC_BF16X3 1     /* pair-factorised coupling + tcgen05 BF16 hi/lo x3 */
#define TP3_MODE_TC_TF32X3 2     /* pair-factorised coupling + tcgen05 TF32 hi/lo x3 */
/* At lambda != 0 the tensor-core modes contract over Fourier pairs (m2, m3): the coupling
 * also writes FP32 T, a SIMT kernel forms H[ki][(m2, m3)] = sum_j T w_j Y1 Y2 Y3 with the
 * shells' Legendre factors (src/correlations.jl:137-148), and the persistent tcgen05
 * kernel contracts H with cos(m2 alpha + m3 beta) on the full N x 2N grid; ragged
 * batches and the per-tile angular schedule above 512 grid points need lambda = 0. */
#define TP3_MODE_AUTO (-1)       /* fastest available mode for this shape */

typedef struct tp3_ctx tp3_ctx;
typedef struct tp3_mlp tp3_mlp;

/* Text for a status code (static storage). */
const char* tp3_status_string(int status);
/* Detail of the last failing call on ctx (or of the last failed tp3_ctx_create
 * on this thread when ctx is NULL). */
const char* tp3_last_error(const tp3_ctx* ctx);
/* ABI version, (major << 16) | minor. */
int tp3_version(void);

/* ---- host-only helpers (no GPU needed) ---------------------------------- */
/* Wigner 3j symbol (j1 j2 j3; m1 m2 m3): role of gsl_sf_coupling_3j as used by
 * wigner() at src/spherical_harmonics.jl:63-65 (argument order here is the
 * symbol's: j1, j2, j3, m1, m2, m3). */
double tp3_wigner3j(int j1, int j2, int j3, int m1, int m2, int m3);
/* sphPlm(l, m, theta): src/spherical_harmonics.jl:69-76. */
double tp3_sphPlm(int l, int m, double theta);
/* Basis sizes without a GPU: info[0] = basislen, [1] = n_lt, [2] = klength,
 * [3] = grid points 2N^2, [4] = unique grid points evaluated, [5] = their
 * multiplicity, [6] = compact coefficients per shell, [7] = entries whose
 * Legendre product is non-zero at theta = pi/2 (lambda = 0).  calculate_basis,
 * src/correlations.jl:87-131. */
int tp3_basis_info(int L, int LMAX, int N, int K, double lambda, double dq, int64_t* info);

/* ---- context ------------------------------------------------------------ */
/* Build tables for (L, LMAX, N, K, lambda, dq) and upload them to the current
 * CUDA device.  lrange = 0:2:L; LMAX >= L+1. */
int tp3_ctx_create(int L, int LMAX, int N, int K, double lambda, double dq, tp3_ctx** out);
void tp3_ctx_destroy(tp3_ctx* ctx);
/* Launch on this cudaStream_t from now on (NULL = the context's own stream). */
int tp3_set_stream(tp3_ctx* ctx, void* cuda_stream);
int tp3_set_mode(tp3_ctx* ctx, int mode);
int tp3_get_mode(const tp3_ctx* ctx, int* mode);

/* Autotuner (no reference counterpart): times, on n synthetic real-function
 * proposals scored against the context's histogram, every evaluation variant this
 * shape supports -- the plain FP32 path and each tensor-core split mode (BF16 x3,
 * TF32 x3) with each coupling form that fits (0: one-kernel pair coupling, 512 threads
 * and up to 225 KB of shared memory per CTA; 2: the same with 256 threads and 110 KB so
 * two CTAs share an SM; 3: warp-local one-kernel coupling, warps taking (k1, k2-quad)
 * units from a counter with no CTA barrier, 512 threads; 4: the warp-local coupling
 * with 256 threads, two CTAs per SM in 110 KB each where that fits, else one with up
 * to 225 KB; 1: two-kernel split coupling through global memory; 5, 6, 7: folded-row
 * coupling, warps owning folded pairs of k1 rows, at 8, 7 and 13 warps per CTA with the
 * largest per-warp D buffer that fits 225 KB; 8: the same at 14 warps in pairs, the two
 * warps of a pair sharing one unit and one D buffer (7 buffers); in BF16 mode it writes
 * T order-major and the angular kernel reads it MN-major) -- selects
 * the fastest for this context and records it for the shape (L, LMAX, N, K, lambda,
 * dq) in the process, where TP3_MODE_AUTO finds it.  Every variant is timed with the
 * persistent angular schedule; the fastest tensor-core variant is then timed again
 * with one CTA per angular tile, and the faster schedule is kept.  report (nullable):
 * up to *nreport rows of four values (mode, coupling form, angular schedule, ms per
 * proposal); *nreport returns the number of rows.  Synchronises. */
int tp3_autotune(tp3_ctx* ctx, int n, double* report, int* nreport);
/* Force a coupling form of the tensor-core path (0 to 8 as above). */
int tp3_set_coupling(tp3_ctx* ctx, int form);
/* Angular-stage schedule of the tensor-core path (no reference counterpart).
 * TP3_ANGULAR_PERSISTENT (default): one CTA per SM walks (proposal, 128-triple tile,
 * grid half) units with two TMEM accumulators, so the Bayes epilogue of one unit
 * overlaps the tensor-core work of the next.  TP3_ANGULAR_TILE: one CTA per
 * (tile, proposal), both grid halves in sequence.  Energies agree to FP32 rounding of
 * the partial sums; the c3 output path always uses the per-tile kernel. */
#define TP3_ANGULAR_TILE 0
#define TP3_ANGULAR_PERSISTENT 1
int tp3_set_angular(tp3_ctx* ctx, int schedule);
/* Pre-size scratch for batches of up to n proposals (otherwise sized on first use). */
int tp3_reserve(tp3_ctx* ctx, int n);

/* Reference histogram c3ref (loadHistograms output).  Slabs are L1-normalised per
 * (k1, k2, k3) exactly as energy() does before the log-likelihood. */
int tp3_set_histogram(tp3_ctx* ctx, const double* c3ref, int K3);

/* Raw model correlation c3 (2N^2 x klength, column-major float). */
int tp3_c3(tp3_ctx* ctx, const double* coeff, float* out);

/* Raw c3 of n coefficient sets in device memory (layout of tp3_energy_batch_device)
 * into d_c3 = n x klength x 2N^2 floats in device memory (per set, the tp3_c3 layout).
 * Asynchronous on the context stream. */
int tp3_c3_batch_device(tp3_ctx* ctx, int n, const void* d_coeffs, void* d_c3);

/* Rotation-invariant triple products T[ki][lt] = sum_{j in lt} w_j Re(c_k1 c_k2 c_k3)
 * (klength x n_lt row-major float) with the current mode's coupling kernel: the
 * As values of calculate_triple_products_fast, src/correlations.jl:157-176. */
int tp3_triple_products(tp3_ctx* ctx, const double* coeff, float* out);

/* Bayes energy of one coefficient set. */
int tp3_energy(tp3_ctx* ctx, const double* coeff, double* E);
/* Bayes energies of n coefficient sets stored back to back (n * K * LMAX^2 complex).
 * Where the device reads pageable host memory through the host page tables (Grace
 * systems with NVLink-C2C), a kernel fetches the coefficients the path uses (even
 * l <= L) straight from coeffs; elsewhere the host packs them into pinned memory and
 * copies them (tp3_set_host_input chooses).  coeffs must stay valid until the call
 * returns, which it does after the energies are in E. */
int tp3_energy_batch(tp3_ctx* ctx, int n, const double* coeffs, double* E);
/* How tp3_energy_batch reaches host coefficients (no reference counterpart):
 * TP3_HOST_INPUT_DIRECT (default where the device supports it) or TP3_HOST_INPUT_STAGED
 * (host packing + one pinned copy).  Both give identical energies. */
#define TP3_HOST_INPUT_STAGED 0
#define TP3_HOST_INPUT_DIRECT 1
int tp3_set_host_input(tp3_ctx* ctx, int mode);
/* Same with device pointers: d_coeffs = n * K * LMAX^2 complex doubles in device
 * memory, d_E = n doubles in device memory.  Asynchronous on the context stream. */
int tp3_energy_batch_device(tp3_ctx* ctx, int n, const void* d_coeffs, void* d_E);

/* ---- ragged batches (no reference counterpart) --------------------------------
 * Proposals of different (L, K) scored in one launch on the context's shape (its L
 * and K are the largest): orders l > L and shells k > K of a proposal are treated as
 * absent -- exactly the reference's c3 of basis (L, K), whose shell triples are the
 * first K(K+1)(K+2)/6 of the context's -- and each proposal is scored against its own
 * histogram of a set.  Tensor-core modes with the one-kernel coupling only. */
/* Histogram set: nhist histograms (each as for tp3_set_histogram, with K3s[h] >= Ks[h]
 * shells stored and Ks[h] <= the context's K scored). */
int tp3_set_histograms(tp3_ctx* ctx, int nhist, const double* const* c3refs, const int* K3s, const int* Ks);
/* Energies of n proposals (d_coeffs as for tp3_energy_batch_device) with per-proposal
 * (L, K, histogram index) triples d_lkh (n x 3 int32, device).  Out-of-range triples
 * are clamped and reported by the next synchronising call as TP3_ERR_ARG. */
int tp3_energy_batch_ragged_device(tp3_ctx* ctx, int n, const void* d_coeffs, const int* d_lkh, void* d_E);
/* Upload per-proposal (L, K, histogram) limits without scoring (used by chains). */
int tp3_ragged_limits_device(tp3_ctx* ctx, int n, const int* d_lkh);

/* Wait for the context stream and report any device-side error (TP3_ERR_TIMEOUT
 * when a bounded wait inside a kernel ran out). */
int tp3_sync(tp3_ctx* ctx);

/* ---- device-resident annealing chains ------------------------------------- */
/* nchains independent simulated-annealing chains of the reference's plain method
 * (rotate_all_at_once + evaluate_step, src/determination.jl:281-338, 491-515),
 * state kept on the device.  Move: get_MC_step (src/determination.jl:232-241) --
 * one random plane rotation by N(0, sigma_l) per even l in 2..L, applied to every
 * shell.  Step sizes start at initial_stepsize * (l - 1) (src/determination.jl:295)
 * and are multiplied (accept) or divided (reject) by stepsizefactor; T decays by
 * temperature_decay before each step; a step is accepted when dE < 0 or when
 * dE > 0 and u < exp(-dE/T) (src/determination.jl:497-509).
 * Each tp3_chains_run launch scores ncand speculative steps per chain in one
 * batch (candidate i assumes the i previous ones were rejected) and advances every
 * chain to its first accepted candidate, so the trajectory is the sequential
 * chain's for the same random numbers (Philox4x32-10, counter = step, chain,
 * purpose, index; key = seed), independent of ncand.  One launch is one replay of
 * a captured CUDA graph.
 *   coeff0: nchains x K x LMAX^2 complex (the layout of tp3_energy_batch)
 *   T0:     nchains initial temperatures (calculate_temperature's result)
 *   log_capacity: per-chain ring of the last steps' det.out columns (0 = none). */
typedef struct tp3_chains tp3_chains;
int tp3_chains_create(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                      double initial_stepsize, double stepsizefactor, double temperature_decay, uint64_t seed,
                      int log_capacity, tp3_chains** out);
/* Chains of different (L, K) scored together (no reference counterpart): chain c
 * uses chain_lkh[3c..3c+2] = (L, K, histogram index of the context's set,
 * tp3_set_histograms), with L <= the context's L (the move rotates orders 2..L) and
 * K <= the histogram's K; all chains' candidates go through one ragged launch per
 * step.  Other arguments as tp3_chains_create; coeff0 holds the context's K shells
 * per chain (shells beyond a chain's K are carried along unscored). */
int tp3_chains_create_ragged(tp3_ctx* ctx, int nchains, int ncand, const double* coeff0, const double* T0,
                             double initial_stepsize, double stepsizefactor, double temperature_decay,
                             uint64_t seed, int log_capacity, const int* chain_lkh, tp3_chains** out);
void tp3_chains_destroy(tp3_chains* chains);
/* Enqueue `launches` graph replays (ncand speculative steps per chain each). */
int tp3_chains_run(tp3_chains* chains, int launches);
/* Synchronise and read E, T, step sizes (nchains x (L/2+1), index l/2), steps
 * taken and steps accepted per chain; any pointer may be NULL. */
int tp3_chains_state(tp3_chains* chains, double* E, double* T, double* sigma, int64_t* steps, int64_t* accepted);
/* Current coefficients, nchains x K x LMAX^2 complex. */
int tp3_chains_coeff(tp3_chains* chains, double* coeff);
/* Last min(steps, log_capacity) steps of one chain, 8 doubles per row: step, sign,
 * E_new, E, dE, T, acceptance probability, sigma_L. */
int tp3_chains_log(tp3_chains* chains, int chain, double* rows, int64_t* nrows);
/* Checkpoint: with buf NULL, *bytes receives the size; otherwise the chain state
 * (coefficients, E, T, counters, step sizes, the network's history inputs) is
 * written to buf.  Restore is bit-exact; the RNG needs no state beyond the step
 * counters. */
int tp3_chains_snapshot(tp3_chains* chains, void* buf, size_t capacity, size_t* bytes);
int tp3_chains_restore(tp3_chains* chains, const void* buf, size_t bytes);
/* Move of a chain set.  TP3_MOVE_REFERENCE (default): get_MC_step
 * (src/determination.jl:232-241).  TP3_MOVE_SHELL_SO3: every shell rotated by its own
 * exp([v]x), v ~ N(0, sigma^2 I3), with the Wigner-D rotation of rotateStructure
 * (src/spherical_harmonics.jl:595-603) on every even l; sigma starts at sigma0 and
 * is multiplied / divided by the step-size factor on accept / reject like the
 * reference's step sizes.  Every launch of per-shell moves also estimates, per chain
 * and shell, the energy gradient from its B candidates (all drawn at the launch's
 * start state):  e_k = (1/B) sum_i ((dE_i - mean_j dE_j) / T) w_ik,  w_ik the
 * candidate's whitened step noise (z for an isotropic step; see below), T the first
 * candidate's temperature; the last 8 launches' e_k are features of the network.
 * TP3_MOVE_LEARNED: a candidate comes from the network (tp3_mlp) with probability
 * p_net and from the isotropic step otherwise.  A network candidate with outputs
 * (u_k, s_k) draws a = +-1 (equally likely) and
 *     v_k = sigma_i (a sqrt(16) u_k / sqrt(sum_k |u_k|^2 + 0.01) + exp(s_k - mean_k s_k) z_k),
 * z_k ~ N(0, I3) (whitened noise exp(-(s_k - mean s)) z_k): a two-sided drift along
 * the network's gradient estimate.  Per-shell steps draw z (and a) from a stream keyed
 * by the chain's launch count, so every launch's candidates carry fresh noise and a
 * per-shell chain's trajectory depends on the candidates per launch (the reference
 * move's draws are keyed by the step and do not).  The Metropolis-Hastings ratio of the mixture
 * density (the network part a two-component mixture over a, evaluated at x' for the
 * reverse step with the network re-run there) corrects the acceptance.  The network
 * must have n_in = (L+1)^2 + 33 and max_rows >= chains x candidates x K.
 * TP3_MOVE_DRIFT: the same mixture with probability p_net and no network: u_k = the
 * chain's newest gradient estimate e_k, all s_k = 0.  The drift is a fixed parameter of
 * the step, so the proposal is symmetric and plain Metropolis acceptance is exact (net
 * is ignored).  It measures what a trained network adds over its own strongest input.
 * No reference counterpart for the three per-shell kinds. */
#define TP3_MOVE_REFERENCE 0
#define TP3_MOVE_SHELL_SO3 1
#define TP3_MOVE_LEARNED 2
#define TP3_MOVE_DRIFT 3
int tp3_chains_set_move(tp3_chains* chains, int kind, double sigma0, double p_net, tp3_mlp* net);

/* Move log for training the network: a ring of `launches` launches of per-shell
 * moves; per candidate the state's feature rows, the steps v, and
 * (dE, T, accepted, drawn-from-network, log q(x|x') - log q(x'|x), sigma_i,
 *  (dE - mean over the launch's candidates of dE) / T) where accepted is the
 * Metropolis decision with the candidate's own uniform (the chain's actual decision
 * up to its taken step) and sigma_i the candidate's isotropic step size.
 * tp3_chains_move_log_count returns the candidates held (synchronising);
 * tp3_chains_move_log_gather writes, for n candidate positions d_idx (int64, device,
 * each < count), n x K feature rows (BF16, stride (L+1)^2 + 33 rounded up to 32, the
 * temperature column set to the candidate's), n x K x 3 steps divided by sigma_i
 * (float) and n x 7 meta floats in that order into device buffers. */
int tp3_chains_enable_move_log(tp3_chains* chains, int launches);
int tp3_chains_move_log_count(tp3_chains* chains, int64_t* candidates);
int tp3_chains_move_log_gather(tp3_chains* chains, int n, const int64_t* d_idx, void* d_x, float* d_v, float* d_meta);

/* *captured = 1 when launches replay a CUDA graph. */
int tp3_chains_graph(const tp3_chains* chains, int* captured);

/* ---- scoring without device allocation ------------------------------------ */
/* No counterpart in the reference.  Bayes energy of a model correlation that is
 * already in device memory, for callers that may not allocate device memory at the
 * time they score: a Julia host whose CUDA.jl memory pool owns the device memory (a
 * foreign cudaMalloc can fail against the pool and synchronises the device inside the
 * annealing loop), runtimes that work within a device-memory budget granted up front,
 * and loops that must not stall on cudaMalloc/cudaFree's implicit synchronisation.
 * The call allocates nothing and needs no context:
 *   d_c3   [klength][2N^2] float, device: c3 in tp3_c3's layout;
 *   d_qhat [klength][2N^2] float, device: histogram slabs, each L1-normalised;
 *   d_E    1 double, device: the energy (src/correlations.jl:201-226);
 *   stream cudaStream_t to launch on (NULL = legacy default stream).
 * klength = K(K+1)(K+2)/6 must be <= 65536 (K <= 72): per-slab partials go to a
 * fixed 512 KiB array in the library's device memory that every GPU which loads
 * the library keeps until the process exits; larger K is rejected with
 * TP3_ERR_ARG.  Set-up: the first call in each CUDA context looks up that array's
 * device address (cudaGetSymbolAddress, which also loads the library's module into
 * the context); make that first call before any stream capture.  The address is
 * looked up again when the calling thread's current context changes (a device reset
 * makes a new one).  All calls share the array: calls whose kernels overlap on the
 * GPU (other streams, other host threads) race on it and must be serialised by the
 * caller.  Each call writes every entry it reads, so no clearing is needed.
 * Asynchronous; errors in the arguments return at once, and a CUDA error left
 * pending by earlier work is reported as such without launching (detail in
 * tp3_last_error(NULL)). */
int tp3_bayes_energy_noalloc(const float* d_c3, const float* d_qhat, int K, int N, double* d_E, void* stream);

/* ---- triplet histograms of photon pictures (src/datagen.jl:228-277) ---------- */
/* histogramCorrelationsInPicture_alltoall for n pictures at once: picture p holds the
 * photons d_photons[d_offsets[p] .. d_offsets[p+1]) (device, n_photons (x, y) detector
 * doubles, the reference's photon vectors with z = 0; d_offsets int64, device; a
 * picture whose range leaves [0, n_photons] is skipped and reported as TP3_ERR_ARG by
 * the next synchronising call).  Adds EXACT
 * entry counts to the device histograms (unsigned 64-bit, the reference's Julia
 * layouts, column-major): c1[K2], c2[N, K2, K2] (ai, k2, k1), c3[N, 2N, K3, K3, K3]
 * (ai, bi, k3, k2, k1).  The reference's weighted histograms are count / k1,
 * count / (doubletFactor k1 k2), count / (tripletFactor k1 k2 k3).  At most 1536
 * photons per picture survive the k filter; a larger picture is skipped and reported
 * as TP3_ERR_ARG by the next synchronising call.  Asynchronous on the context stream. */
int tp3_histogram_pictures(tp3_ctx* ctx, int n_pictures, const void* d_photons, int64_t n_photons,
                           const int64_t* d_offsets, double dq, int N, int K2, int K3, unsigned long long* d_c1,
                           unsigned long long* d_c2, unsigned long long* d_c3);
/* pointsPerOrientation (src/datagen.jl:88-144) for pictures first_picture ..
 * first_picture + n_pictures - 1 of an intensity given by SH coefficients d_coeff
 * (KMAX x LMAX^2 complex128, seanindex order, shell k at |q| = k dq, linear in |q|
 * between shells): a Haar-random orientation per picture, incident_photons Gaussian
 * detector photons of width envelope_sigma, those with |p| <= qcut mapped to the Ewald
 * sphere (wavelength lambda) and kept with probability
 * I(R e(p)) exp(|e(p)|^2 / (2 sigma^2)) / max_intensity.  Accepted (x, y) go to
 * d_photons[p][0 .. d_counts[p]) (n_pictures x max_out double pairs, device).
 * Philox4x32-10 streams keyed by seed (independent of how pictures are batched). */
int tp3_sample_pictures(tp3_ctx* ctx, int n_pictures, int64_t first_picture, const void* d_coeff, int KMAX, int LMAX,
                        double dq, double qcut, double envelope_sigma, int incident_photons, double lambda,
                        double max_intensity, uint64_t seed, int max_out, void* d_photons, int* d_counts);
/* pointsPerOrientation with the rest of generateHistogram's picture model
 * (src/datagen.jl:88-113, 397-405): as tp3_sample_pictures, plus
 *   incident_photon_variance > 0: the picture's incident photons are
 *     round(N(incident_photons, incident_photon_variance)) (the reference passes it as
 *     the standard deviation of its Normal), clamped to 0 .. 2^24;
 *   beamstop_width > 0: incident photons with |x| <= beamstop_width or
 *     |y| <= beamstop_width are dropped before the qcut test;
 *   stream (0..15): independent photon draws for the same pictures and orientations
 *     (0 molecule; GaussianNoise photons are a second call with stream 1, the noise
 *     intensity and the envelope width noise.sigma * 1.05). */
int tp3_sample_pictures_ex(tp3_ctx* ctx, int n_pictures, int64_t first_picture, const void* d_coeff, int KMAX,
                           int LMAX, double dq, double qcut, double envelope_sigma, int incident_photons,
                           int incident_photon_variance, double beamstop_width, int stream, double lambda,
                           double max_intensity, uint64_t seed, int max_out, void* d_photons, int* d_counts);
/* Largest intensity on the shells x (n_theta x n_phi) grid (the maximum the
 * rejection sampling is normalised by).  Synchronises. */
int tp3_intensity_max(tp3_ctx* ctx, const void* d_coeff, int KMAX, int LMAX, double dq, int n_theta, int n_phi,
                      double* out);

/* ---- structure -> SH coefficients (src/structure.jl:125-134) ------------------
 * FP64 on the context's device and stream, for n_mol molecules at once.  atoms:
 * [n_atoms][5] = x, y, z (Angstrom, centred as centerStructure does), R, B (the atom
 * factor of its element, src/structure.jl:8-16); molecule i owns atoms mol_start[i] ..
 * mol_start[i + 1] - 1 (mol_start[0] = 0).  Each shell is sampled on the reference's
 * surface grid (getSurface / i_to_ang: 2 LMAX x 2 LMAX points) and transformed with the
 * semantics of the s2kit forward transform at bandwidth LMAX (transform,
 * src/spherical_harmonics.jl:127-136): orthonormal Y_lm with the Condon-Shortley phase,
 * coefficients in seanindex order.  Outputs (host, nullable) are [n_mol][KMAX][LMAX^2]
 * complex (re, im interleaved); shell k (1-based) of the density sits at
 * r = k rmax / KMAX, of the amplitude and intensity at q = k pi / rmax.
 *   TP3_SH_INTENSITY: intensity = transform of |F(q)|^2 (getIntensity_cartesian,
 *     src/structure.jl:89-102), the reference's intensityShell route; density and
 *     amplitude must be NULL.
 *   TP3_SH_REFERENCE: the route of createSphericalHarmonicsStructure: density shells
 *     (getDensity_cartesian, atoms cut at |x - a|^2 < 5) -> transform -> forward
 *     spherical Bessel transform (sphBesselTransform, src/spherical_harmonics.jl:291-347)
 *     = amplitude -> absoluteSquare (src/spherical_harmonics.jl:376-381) = intensity.
 * 2 <= LMAX <= 48, 2 <= KMAX <= 4096.  Synchronises. */
#define TP3_SH_INTENSITY 0
#define TP3_SH_REFERENCE 1
int tp3_structure_sh(tp3_ctx* ctx, const double* atoms, const int* mol_start, int n_mol, int LMAX, int KMAX,
                     double rmax, int route, double* density, double* amplitude, double* intensity);

/* Post-processing fit, fitStructures_random (src/data_processing.jl:51-75), on the
 * context's device for a structure of the context's shape: volume and reference are host
 * [K][LMAX^2] complex (seanindex order); shells k_lo..k_hi (1-based) are scored.  Each of
 * `repetitions` random restarts walks rotations rotationMatrix(theta, phi, gamma) of orders
 * 2:2:L, step size pi shrunk by stepsizefactor (0 < f < 1) per step while it exceeds one
 * degree (S steps), and keeps a proposal whose similarity -- the mean over the shells of the
 * Pearson correlation of the two intensities on the synthesis grid of transform /
 * backtransform (2 LMAX x 2 LMAX) -- beats its best.  draws: [repetitions][3 + 3 S]: three
 * uniforms in [0, 1) for the start (phi = 2 pi u0, theta = acos(u1), gamma = 2 pi u2), then
 * per step three standard normals (theta += n0 step / 2, phi += n1 step, gamma += n2 step).
 * best (out): similarity, theta, phi, gamma of the best restart (the first on ties).
 * rotated (nullable): [K][LMAX^2] complex, the volume with shells 1..k_hi rotated by it.
 * FP64.  Synchronises. */
int tp3_fit_structures_random(tp3_ctx* ctx, const double* volume, const double* reference, int k_lo, int k_hi, int L,
                              double stepsizefactor, int repetitions, const double* draws, double* best,
                              double* rotated);

/* retrieveSolution (src/correlations.jl:261-319): intensity coefficients consistent with
 * a two-photon correlation, on the context's device.  c2: host [N][Kd][Kd] doubles,
 * c2[alpha][k2 - 1][k1 - 1] as twoPhotons writes it; shells k_lo..k_hi (K2 = k_hi - k_lo + 1
 * <= 64, L even with 2 L < K2), dq = qmax / k_hi.  Per shell pair a least-squares fit of
 * the slice (symmetrised in alpha at lambda = 0) on (1/4pi) P_l(cos alpha*), l = 0:2:upperL,
 * upperL = min(L, 2 min(k1, k2) - 2), gives G_l[k1, k2]; the top 2l+1 eigenpairs of each
 * G_l (eigenvector signs fixed by making the largest entry positive) give real SH
 * coefficients sqrt(w) v^T, mapped to complex ones with Umat(l)^*; the whole structure is
 * negated when negativityCheck on the synthesis grid exceeds 0.33.  out: host [k_hi][LMAX^2]
 * complex (shells below k_lo zero).  FP64.  Synchronises. */
int tp3_retrieve_solution(tp3_ctx* ctx, const double* c2, int N, int Kd, int L, int LMAX, int k_lo, int k_hi,
                          double qmax, double lambda, double* out);

/* ---- Wigner-D rotations (src/spherical_harmonics.jl:572-603) --------------- */
/* rotationMatrix(theta, phi, gamma, l) of src/spherical_harmonics.jl:590-592:
 * D[m, s] = exp(-i s gamma - i m phi) d^l_{ms}(theta), m, s = -l..l, written
 * column-major (Julia order) as (2l+1)^2 interleaved (re, im) doubles.  It is the
 * coefficient action of the rotation R = Rz(phi) Ry(-theta) Rz(gamma) on functions
 * (f'(n) = f(R^T n)).  Host only, FP64; l <= 62. */
int tp3_wigner_D(int l, double theta, double phi, double gamma, double* out);

/* Per-shell rotations on the device: every shell k of n coefficient sets
 * (d_coeffs / d_out: n x K x LMAX^2 complex128, the layout of
 * tp3_energy_batch_device; d_out may equal d_coeffs) is replaced by
 * rotateStructure's D c_l (src/spherical_harmonics.jl:595-603) for every
 * l < LMAX, with its own rotation exp([v]x), v = d_axis_angle[set][k][0..2]
 * (n x K x 3 doubles, axis times angle in radians): the coefficients of
 * f'(n) = f(R^T n).  rotationMatrix(theta, phi, gamma) is that action for
 * R = Rz(phi) Ry(-theta) Rz(gamma); the Euler angles are taken from exp([v]x).
 * FP64; asynchronous on the context stream.  No reference counterpart as one call:
 * the reference rotates one volume at a time on the host. */
int tp3_rotate_shells_device(tp3_ctx* ctx, int n, const void* d_coeffs, const void* d_axis_angle, void* d_out);

/* ---- learned proposal network ------------------------------------------------
 * No reference counterpart: the network that proposes per-shell rotation steps for
 * the annealer (a mixture with the isotropic step, Metropolis-Hastings corrected).
 * Architecture: n_in -> hidden -> hidden -> hidden -> 6, ReLU, BF16 weights and
 * activations, FP32 accumulation on the tensor cores, FP32 master weights and
 * Adam.  Rows are shells; input rows are BF16 with a stride of n_in rounded up to
 * 32 (the padding columns must be zero).  Outputs per row: u[3] (the shell's drift
 * direction: an estimate of sigma g / T, g the energy gradient of the shell's rotation)
 * and s[3] (log of the step's standard deviation in units of sigma, in (-7, 1)).
 * Parameters are one FP32 vector: W1 (hidden x n_in, row-major), b1, W2, b2, W3, b3,
 * W4 (6 x hidden), b4. */
int tp3_mlp_create(tp3_ctx* ctx, int n_in, int hidden, int max_rows, uint64_t seed, tp3_mlp** out);
void tp3_mlp_destroy(tp3_mlp* net);
int tp3_mlp_num_params(const tp3_mlp* net, int64_t* count);
int tp3_mlp_get_params(tp3_mlp* net, float* host, int64_t count);
int tp3_mlp_set_params(tp3_mlp* net, const float* host, int64_t count);
/* The network's own input buffer (max_rows x row_stride BF16, device): writing the
 * features there saves the copy that the calls below make from any other pointer. */
int tp3_mlp_input_buffer(tp3_mlp* net, void** d_x, int* row_stride);
/* (u, s) of rows [0, rows) into d_out = rows x 6 floats (device).  Asynchronous. */
int tp3_mlp_forward_device(tp3_mlp* net, int rows, const void* d_x, void* d_out);
/* Training loss of logged candidates, `shells` consecutive rows each, steps d_v
 * (rows x 3 floats, v / sigma):
 *   sum_j lambda_j (t_j - sum_k u_k . v_k)^2 / 2            (d_target = (t_j, lambda_j)
 *                                                           per candidate, rows/shells
 *                                                           float pairs; NULL: no term)
 * + sum_r w_r sum_d [s_d + v_d^2 exp(-2 s_d) / 2 + log(2 pi) / 2]   (weights d_w, rows)
 * and its gradient (FP32, the parameter layout) copied to grad_host when not NULL.
 * rows must be a multiple of 128 (pad with w = 0, lambda = 0 and zero features).
 * Synchronises. */
int tp3_mlp_loss_grad(tp3_mlp* net, int rows, const void* d_x, const float* d_v, const float* d_w,
                      const float* d_target, int shells, double* loss, float* grad_host);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on that loss; the loss is returned
 * (synchronising) when loss is not NULL, else the call stays asynchronous. */
int tp3_mlp_train_step(tp3_mlp* net, int rows, const void* d_x, const float* d_v, const float* d_w,
                       const float* d_target, int shells, float lr, double* loss);

/* ---- failure detection self test (no reference counterpart) ------------------- */
/* Launch a kernel whose bounded mbarrier wait can never complete, with a limit of
 * `cycles` SM clocks (1e3 .. 4e9): the wait runs out, the kernel records
 * TP3_ERR_TIMEOUT and returns, and the next synchronising call on the context
 * (tp3_sync, tp3_energy*, ...) reports TP3_ERR_TIMEOUT; the context stays usable. */
int tp3_selftest_timeout(tp3_ctx* ctx, long long cycles);

/* ---- per-launch timing of the stages ------------------------------------- */
/* When enabled, CUDA events bracket each launch of the angular + Bayes kernel and
 * (tensor-core modes) of the coupling kernel on the launching stream;
 * tp3_profile_read_stage(stage 0 = angular, 1 = coupling) returns that stage's launch
 * count and summed milliseconds (synchronising the stream) and resets both;
 * tp3_profile_read is stage 0. */
int tp3_profile_enable(tp3_ctx* ctx, int on);
int tp3_profile_read(tp3_ctx* ctx, int64_t* launches, double* total_ms);
int tp3_profile_read_stage(tp3_ctx* ctx, int stage, int64_t* launches, double* total_ms);

/* ---- measured FP32 peak (the coupling stage's roofline denominator) ------------
 * Times a kernel of independent FP32 FMA chains filling every SM (8 chains per
 * thread, 2048 threads per SM) with CUDA events on the context stream and returns the
 * best of three runs in TFLOP/s (2 flops per FMA).  Synchronises.  No reference
 * counterpart. */
int tp3_measure_fp32_peak(tp3_ctx* ctx, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* TP3_H */
