/*
 * boss.h -- C ABI of libboss_gb300.so, the GB300 (sm_103a) implementation of
 * theboss's permanent hot path.
 *
 * theboss is pure Python and has no FFI of its own; each entry point below
 * replaces one Python-level interface of the reference (cited per function,
 * paths inside the theboss project) and is what a ctypes / cffi binding in that
 * project would bind.
 *
 * Conventions shared by every entry point:
 *   - matrices are complex128 (two doubles per entry, real then imaginary),
 *     row-major m x m, indexed U[output_mode][input_mode] exactly as theboss
 *     indexes them (ryser_permanent_calculator.py:62-64);
 *   - occupation vectors are int32, length `len` (len <= m), mode-occupation
 *     ("second quantisation") form;
 *   - every pointer is a HOST pointer; the library copies to and from the GPU
 *     itself and returns only after the results are back in host memory;
 *   - the return value is a status code (BOSS_OK = 0); boss_last_error() gives a
 *     one-line message for the calling thread;
 *   - calls are serialised by an internal mutex; all GPU work runs on one
 *     library-owned CUDA stream of the current device.
 */
#ifndef BOSS_GB300_H
#define BOSS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BOSS_ABI_VERSION 1

#if defined(__GNUC__)
#define BOSS_API __attribute__((visibility("default")))
#else
#define BOSS_API
#endif

/* Status codes. */
#define BOSS_OK 0
#define BOSS_ERR_SIZE 1      /* size mismatch; theboss raises AttributeError (bs_permanent_calculator_base.py:179-180) */
#define BOSS_ERR_LIMIT 2     /* beyond this library's limits (distinct modes, code count) */
#define BOSS_ERR_CUDA 3      /* CUDA runtime failure */
#define BOSS_ERR_ARG 4       /* invalid argument */
#define BOSS_ERR_PMF 5       /* a sampling pmf could not be normalised; theboss raises ValueError
                                from numpy.random.choice (generalized_cliffords_b_simulation_strategy.py:107-110) */
#define BOSS_ERR_NODEVICE 6  /* no CUDA device */

/* Permanent formulas (bs_permanent_calculator_factory.py:29-33). */
#define BOSS_CLASSIC 3   /* classic_permanent_calculator.py:18-67 semantics (zero-particle rules), Glynn sweep */
#define BOSS_GLYNN 2     /* glynn_gray_permanent_calculator.py:27-84 */
#define BOSS_CHIN_HUH 1  /* chin_huh_permanent_calculator.py:18-59 */
#define BOSS_RYSER 0     /* ryser_permanent_calculator.py:19-64 */

/* Message of the last failed call on this thread (empty if none). */
BOSS_API const char* boss_last_error(void);

/* BOSS_ABI_VERSION of the loaded library. */
BOSS_API int boss_abi_version(void);

/* Binds the library to a CUDA device (call before any other GPU entry point; one
 * process drives one GPU).  Without it the library uses the current device. */
BOSS_API int boss_select_device(int32_t device);

/* Number of SMs of the current device (also initialises the library's context). */
BOSS_API int boss_device_sm_count(int32_t* sm_count);

/*
 * Permanents of `count` effective scattering matrices U[T_k, S_k] of one matrix.
 * Replaces BSPermanentCalculatorInterface.compute_permanent
 * (bs_permanent_calculator_interface.py:18-22) of the calculator chosen by
 * `variant` (RyserPermanentCalculator.compute_permanent,
 * bs_permanent_calculator_base.py:166-198; ChinHuhPermanentCalculator, same;
 * GlynnGrayPermanentCalculator.compute_permanent, glynn_gray_permanent_calculator.py:41-71;
 * ClassicPermanentCalculator.compute_permanent, classic_permanent_calculator.py:27-39),
 * batched over the output patterns a sampler or distribution calculator asks for
 * (bs_distribution_calculator_with_fixed_losses.py:127-142).
 *   matrix         : m x m complex128
 *   input_states   : count x len int32 (S_k)
 *   output_states  : count x len int32 (T_k)
 *   results        : count complex128 (2*count doubles)
 */
BOSS_API int boss_perm_batch(const double* matrix, int32_t m, const int32_t* input_states, const int32_t* output_states,
                    int32_t len, int32_t count, int32_t variant, double* results);

/*
 * All-minors permanents: for each k and each input mode i, perm(U[T_k, S_k - e_i])
 * (0 where S_k[i] = 0), in one sweep per k.  Replaces
 * BSSubmatricesPermanentCalculatorInterface.compute_permanents
 * (bs_submatrices_permanent_calculator_interface.py:17-20) of
 * BSCCRyserSubmatricesPermanentCalculator (bs_cc_ryser_submatrices_permanent_calculator.py:16-119)
 * and BSCCCHSubmatricesPermanentCalculator (bs_cc_ch_submatrices_permanent_calculator.py:25-105),
 * including the one-particle edge case (bs_submatrices_permanent_calculator_base.py:157-158).
 *   variant        : BOSS_RYSER or BOSS_CHIN_HUH
 *   results        : count x len complex128
 */
BOSS_API int boss_submatrices_batch(const double* matrix, int32_t m, const int32_t* input_states,
                           const int32_t* output_states, int32_t len, int32_t count, int32_t variant,
                           double* results);

/*
 * Permanents and their gradients with respect to the matrix.  For each k,
 * perms[k] = perm(U[T_k, S_k]) and grads[k][j][i] = d perm / d U[j][i]
 * = T_k[j] * S_k[i] * perm(U[T_k - e_j, S_k - e_i]) (zero where either mode is
 * empty), all from one Glynn sweep per permanent.  theboss has no derivative;
 * its per-minor counterpart is BSCCRyserSubmatricesPermanentCalculator.compute_permanents
 * (bs_cc_ryser_submatrices_permanent_calculator.py:16-119) called once per removed
 * output particle.  Requires sum(S_k) == sum(T_k).
 *   perms : count complex128;  grads : count x len x len complex128 (row = output mode)
 */
BOSS_API int boss_perm_grad_batch(const double* matrix, int32_t m, const int32_t* input_states,
                                  const int32_t* output_states, int32_t len, int32_t count, double* perms,
                                  double* grads);

/*
 * Benchmark form of boss_perm_batch for `count` permanents with the same number
 * of product-side particles: planned and uploaded once, then the sweep kernel and
 * its reduction run n_warmup + n_steps times (an L2-evicting memset of
 * flush_bytes before each).  sweep_ms receives the sweep kernel's CUDA-event time
 * per timed run; info[0..4] = codes swept per run, algorithmic flops per run
 * (codes x (8 nf - 4): nf complex adds, nf - 1 complex products and one signed
 * add per code), threads, nf, and the FP32 instructions per run of the
 * float-pair sweep (codes x (53.125 nf - 22); 0 in FP64).  info must hold 5
 * doubles.  results (optional) receives the permanents.  No reference
 * counterpart.
 */
BOSS_API int boss_perm_bench(const double* matrix, int32_t m, const int32_t* input_states,
                             const int32_t* output_states, int32_t len, int32_t count, int32_t variant,
                             int32_t n_warmup, int32_t n_steps, int64_t flush_bytes, double* sweep_ms, double* info,
                             double* results);

/*
 * The random stream theboss's C&C-B samplers draw, replayed on the host without a
 * GPU.  numpy's legacy global RandomState is an MT19937 generator; its state
 * (numpy.random.get_state(): 624-word key and position) is passed in and
 * returned advanced exactly as theboss's own draws would advance it:
 *   per sample, with particle_weights (uniform losses): one random() compared with
 *   the running sum of the weights (generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-85);
 *   per step: randint(0, remaining) picks the popped particle
 *   (generalized_cliffords_b_simulation_strategy.py:102-105) and one random_sample()
 *   is consumed by numpy.random.choice (:107-110).
 * particle_weights NULL means lossless (every particle kept, no count draw).
 *   particles_kept : n_samples int32
 *   popped_modes   : n_samples x n int32 (n = sum(input_state)); -1 past the kept count; may be NULL
 *   uniforms       : n_samples x n doubles; may be NULL
 */
BOSS_API int boss_gccb_predraw(const int32_t* input_state, int32_t m, const double* particle_weights,
                               int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples,
                               int32_t* particles_kept, int32_t* popped_modes, double* uniforms);

/*
 * n_samples generalized Clifford & Clifford (version B) samples on the GPU.
 * Replaces GeneralizedCliffordsBSimulationStrategy.simulate
 * (generalized_cliffords_b_simulation_strategy.py:41-67) when particle_weights is
 * NULL, and GeneralizedCliffordsBUniformLossesSimulationStrategy.simulate
 * (generalized_cliffords_b_uniform_losses_simulation_strategy.py:87-109) with the
 * binomial particle-number weights (:50-65); LossyNetworksGeneralizedCliffordsSimulationStrategy
 * (lossy_networks_generalized_cliffords_simulation_strategy.py:53-83) is the lossless
 * call on the 2m x 2m expanded matrix.  Consumes numpy's MT19937 stream exactly as
 * boss_gccb_predraw describes and returns the advanced state, so the samples are
 * the ones theboss draws with the same seed (given the same probabilities).
 * All samples run level-synchronously: the all-minors sweeps of every sample at
 * one step in one launch, the whole loop as one CUDA graph.
 *   matrix   : m x m complex128, m <= 256;  sum(input_state) <= 32
 *   samples  : n_samples x m int32 output occupations
 */
BOSS_API int boss_gccb_sample(const double* matrix, int32_t m, const int32_t* input_state,
                              const double* particle_weights, int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos,
                              int32_t n_samples, int32_t* samples);

// Arithmetic of the all-minors sweeps (boss_submatrices_batch and the batched
// sampler's levels, boss_gccb_sample*, boss_gccb_bench; theboss computes them in
// numpy float64, bs_cc_ryser_submatrices_permanent_calculator.py:96-119, and the
// sampler's pmf in Python floats, generalized_cliffords_b_simulation_strategy.py:82-92).
// mode 1 (default): FP64 sweeps, and the sampler's Laplace step, |.|^2 and pmf in
// FP64; mode 0: products, running totals, minors and the sampler's pmf as float
// pairs (two FP32 values, about 47 significant bits) on the FP32 pipe, for
// sweeps of at most 24 product-side particles (larger ones stay FP64); -1: query
// only.  *previous (if not null) receives the mode in force before the call.  Row
// sums are exact 64-bit fixed point in both; in mode 1 the first factors of every
// product are multiplied in block floating point on the integer pipe (62-bit
// mantissas, each product within 2^-56.5 of its magnitude, rounded once to FP64).
BOSS_API int boss_minors_arithmetic(int32_t mode, int32_t* previous);

// The same choice for the single-permanent sweeps of boss_perm_batch and
// boss_perm_bench (theboss: numpy float64 in every calculator's
// compute_permanent, bs_permanent_calculator_base.py:166-198): 1 FP64 (default),
// 0 float pairs (up to 32 product-side particles, Glynn-kind sweeps: Glynn,
// Chin-Huh, Classic), -1 query.  Ryser-form sweeps, whose alternating sum cancels
// far more, the allocation-free entry point and the gradients always use FP64 (in
// the FP64 single-permanent sweeps all but the last 8 factors of every product are
// multiplied in block floating point on the integer pipe, as above).
BOSS_API int boss_perm_arithmetic(int32_t mode, int32_t* previous);

/*
 * The sampler's cdf guard.  Every draw of boss_gccb_sample* is decided from the
 * pmf the GPU computed; when a step of the cdf lies within the pmf's error bound
 * of the uniform (a near tie, where the rounding of the minors could change the
 * outcome), theboss's exact sequential rule on the pmf decides it (Python's sum,
 * the division, numpy's cumsum and searchsorted:
 * generalized_cliffords_b_simulation_strategy.py:91-92, 107-110).  *count receives
 * the number of such draws since the last reset; reset != 0 zeroes the count.
 * No reference counterpart.
 */
BOSS_API int boss_gccb_near_ties(int64_t* count, int32_t reset);

/*
 * The sampler's autotuner.  On the workload of a boss_gccb_sample call (the same
 * arguments; the MT19937 state is read, not advanced) it times, per level of
 * the sampler, power-of-two shifts of the split (threads per sample) and caps of
 * the size of the thread groups that sum their minors inside the sweep, keeps
 * the fastest shape of every level when the whole step gets faster, then times
 * the pipelined parts (the first part's size and the growth of the later ones)
 * on end-to-end calls (calls of at least 4096 samples).  The winners apply to later calls whose levels have the same
 * arithmetic, particle count and power-of-two sample count; they are kept for
 * the process and in a cache file keyed by the GPU's name ($BOSS_TUNE_CACHE, else
 * ~/.cache/theboss_gb300/gccb_tune.txt), which later processes load.  With the
 * environment variable BOSS_AUTOTUNE=1, boss_gccb_sample* tune an untuned
 * workload on its first call.  reps: timed runs per candidate (after one warm-up).
 * report (8 doubles): step ms with the heuristic shapes, step ms with the tuned
 * shapes, levels whose shape changed, the pipeline shift (first part = count >>
 * shift), end-to-end ms with the default parts (shift 4, each later part twice
 * the one before) and with the tuned ones (0 below 4096 samples), the summed
 * per-level times of the heuristic shapes (each level from its sweep's start to
 * its finalize's end; the step time minus this is the time between levels), and
 * the growth factor of the later parts.  No reference counterpart.
 */
BOSS_API int boss_gccb_autotune(const double* matrix, int32_t m, const int32_t* input_state,
                                const double* particle_weights, int32_t n_weights, const uint32_t* mt_key,
                                const int32_t* mt_pos, int32_t n_samples, int32_t reps, double* report);

/*
 * Benchmark form of boss_gccb_sample: the random stream is replayed and the
 * inputs uploaded once, then the captured sampler graph runs n_warmup + n_steps
 * times with inputs resident in GPU memory.  Before every run a flush_bytes
 * memset evicts L2.  Per timed run it writes the graph time (step_ms) and the
 * summed time of its all-minors sweep launches (sweep_ms), both from CUDA events
 * on the library stream.  info[0..6] = flops of the sweeps per run (9k - 12 per
 * Guan code at level k, over the codes the Glynn-form sweeps walk), H2D bytes and
 * D2H bytes of one boss_gccb_sample call, kernels per run, sweep launches per
 * run, the deepest level, the same flop count over theboss's Ryser-form codes
 * (twice as many for single photons), and the FP32 instructions per run of the
 * float-pair sweeps (47.5625 nf per code at nf factors: nf - 1 float-pair
 * complex products of 32, two complex float-pair sums of 16 for the running
 * total and a minor, 31/32 of the codes 16 per factor to move the sums, 1/32 of
 * them 2 per factor to convert; 0 when the sweeps run in FP64).  info must hold 8 doubles.  samples
 * (optional) receives the last run's samples.  No reference counterpart.
 */
BOSS_API int boss_gccb_bench(const double* matrix, int32_t m, const int32_t* input_state,
                             const double* particle_weights, int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos,
                             int32_t n_samples, int32_t n_warmup, int32_t n_steps, int64_t flush_bytes,
                             double* step_ms, double* sweep_ms, double* info, int32_t* samples);

/*
 * Allocation-free form of boss_perm_batch, for callers that cannot let a library
 * call cudaMalloc: processes that give the GPU's memory to their own pool
 * allocator and must account for every byte, services under a hard memory cap,
 * and latency-sensitive loops that avoid cudaMalloc's implicit device
 * synchronisation.  This entry point has no counterpart in theboss.
 *   - It allocates nothing: its scratch (sweep descriptors, fixed-point rows and
 *     per-thread partial sums) is one static 8 MiB device array that every GPU
 *     loading the library holds until the process exits.  A request needing
 *     more scratch is rejected with BOSS_ERR_LIMIT (split the batch).
 *   - matrix and the occupation vectors are host pointers (the sweep is planned
 *     on the host); results_device is a device buffer of `count` complex128 owned
 *     by the caller; work is queued on `stream` (a cudaStream_t, 0 for the
 *     default stream) and the call returns without waiting for it: synchronise
 *     the stream before reading the results.
 *   - The request is planned whole before anything is queued: a rejected
 *     request leaves the caller's buffer untouched.
 *   - The first call on each device does a one-time set-up with that device
 *     current: it looks up the scratch array's device address, sets kernel
 *     attributes and creates one event; the first call in the process also
 *     page-locks the library's 8 MiB host staging array (cudaHostRegister, no
 *     device memory).  Make that first call before any stream capture.
 *   - The host staging array is refilled only after its previous copy has left
 *     it (an event wait), so calls may be queued back to back on one stream.
 *   - Every call shares the scratch array, which keeps the last call's contents;
 *     nothing in it has to start at zero.  Calls on the same stream are ordered;
 *     calls whose work overlaps on the GPU (different streams or threads) race on
 *     the scratch and must not be issued.
 */
BOSS_API int boss_perm_batch_noalloc(const double* matrix, int32_t m, const int32_t* input_states,
                                     const int32_t* output_states, int32_t len, int32_t count, int32_t variant,
                                     double* results_device, void* stream);

/*
 * FP64 throughput of the current GPU: a dependency-free DFMA stream on every SM,
 * timed with CUDA events.  Writes TFLOP/s (an FMA counts 2 flops) and the kernel
 * time.  No reference counterpart: it is the denominator of the FP64 roofline.
 */
BOSS_API int boss_fp64_peak(double* tflops, double* milliseconds);

/*
 * FP32 FMA instruction throughput of the current device (10^12 lane
 * instructions per second) from a stream of independent FFMA chains: the
 * denominator of the float-pair kernels' FP32 roofline.  No reference
 * counterpart.
 */
BOSS_API int boss_fp32_peak(double* tinst, double* milliseconds);

/*
 * Exact probability of each outcome after particle losses, with l = sum(outcome)
 * of the initial state's particles surviving.  Replaces
 * BSDistributionCalculatorWithFixedLosses.__calculate_probability_of_outcome
 * (bs_distribution_calculator_with_fixed_losses.py:84-151) with
 * number_of_particles_left = l, evaluated for all outcomes at once; the
 * uniform-loss calculator (bs_exact_distribution_with_uniform_losses.py:62-97)
 * multiplies by its weight of l.
 *   - outcomes: count x m occupations (any mix of particle counts <= sum(initial));
 *     probabilities: count doubles.
 *   - Lossy inputs in theboss's order (generate_lossy_n_particle_input_states);
 *     an outcome with no particle has probability 1.
 *   - kernel_ms (may be null): GPU time of the per-pair kernels, for benchmarks.
 * BOSS_ERR_ARG when an outcome holds more particles than the initial state;
 * BOSS_ERR_LIMIT beyond 5e7 particle combinations or 8 multiply occupied modes.
 */
BOSS_API int boss_lossy_probabilities(const double* matrix, int32_t m, const int32_t* initial_state,
                                      const int32_t* outcomes, int32_t count, double* probabilities,
                                      float* kernel_ms);

/*
 * How many of the n_samples samples (n_samples x m occupations) equal each of the
 * n_outcomes listed outcomes; a sample equal to several listed outcomes counts for
 * the first.  Replaces the Python scan of
 * BSSampleBasedDistributionCalculator.calculate_approximate_distribution
 * (bs_sample_based_distribution_calculator.py:94-106).  counts: n_outcomes int64.
 * Sample occupations must lie in [0, 254] (BOSS_ERR_ARG otherwise); an outcome
 * outside that range matches no sample.
 */
BOSS_API int boss_count_outcomes(const int32_t* samples, int64_t n_samples, const int32_t* outcomes,
                                 int64_t n_outcomes, int32_t m, int64_t* counts);

/*
 * One lossless C&C-B sample per (matrix, input state) instance, all instances in
 * one batched run.  Replaces the per-sample `helper_strategy.simulate(input)[0]`
 * calls of the BOBS strategies (lossy_state_approximated_simulation_strategy.py:298-310,
 * nonuniform_losses_approximation_strategy.py:274-296) and of
 * GeneralizedCliffordsBSimulationStrategy.simulate (generalized_cliffords_b_simulation_strategy.py:41-110).
 *   - matrices: n_matrices complex m x m (row-major U[out][in]); n_matrices is 1
 *     (shared) or n_samples.  input_states: n_samples x m.
 *   - randint_results / uniforms: n_samples x stride, the numbers theboss draws per
 *     step (randint(0, particles left), then numpy.random.choice's random_sample);
 *     entry k of row s is used for k < sum(input_states[s]).
 *   - samples: n_samples x m output occupations.
 * At most 32 particles per instance (BOSS_ERR_LIMIT); a randint result outside
 * [0, particles left) is BOSS_ERR_ARG; an unnormalisable pmf is BOSS_ERR_PMF.
 */
/*
 * boss_gccb_sample for one slice of a sample stream: replays the whole stream of
 * n_samples samples (advancing the MT19937 state over all of them) and samples
 * only samples [first, first + count) into `samples` (count x m).  Ranks that
 * each take a slice of the same stream, from the same state, together produce
 * exactly the samples of one boss_gccb_sample call (data-parallel sampling with
 * the single-process stream).
 */
BOSS_API int boss_gccb_sample_slice(const double* matrix, int32_t m, const int32_t* input_state,
                                    const double* particle_weights, int32_t n_weights, uint32_t* mt_key,
                                    int32_t* mt_pos, int32_t n_samples, int32_t first, int32_t count,
                                    int32_t* samples);

BOSS_API int boss_gccb_sample_instances(const double* matrices, int32_t n_matrices, int32_t m,
                                        const int32_t* input_states, int32_t n_samples,
                                        const int32_t* randint_results, const double* uniforms, int32_t stride,
                                        int32_t* samples);

/*
 * The random numbers of n_samples samples of the uniform-loss BOBS strategy
 * (LossyStateApproximationSimulationStrategy._simulate_in_parallel,
 * lossy_state_approximated_simulation_strategy.py:287-362), drawn in theboss's
 * order from numpy's legacy MT19937 state (advanced in place): per sample the
 * approximated part (choice over approx_parts with approx_weights), the exact
 * part (choice over exact_parts), m - k phase uniforms, numpy's shuffle of
 * range(m), then the C&C-B steps.  exact_parts: n_exact x k occupations;
 * approx_parts: n_approx x (m - k).  Outputs: input_states (n_samples x m, the
 * stacked parts), phase_uniforms (n_samples x (m - k)), permutations
 * (n_samples x m), randint_results / uniforms (n_samples x stride).
 */
BOSS_API int boss_bobs_uniform_predraw(uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t m, int32_t k,
                                       const int32_t* exact_parts, const double* exact_weights, int32_t n_exact,
                                       const int32_t* approx_parts, const double* approx_weights, int32_t n_approx,
                                       int32_t stride, int32_t* input_states, double* phase_uniforms,
                                       int32_t* permutations, int32_t* randint_results, double* uniforms);

/*
 * The random numbers of n_samples samples of the non-uniform-loss BOBS strategy
 * (NonuniformLossesApproximationStrategy._simulate_in_parallel,
 * nonuniform_losses_approximation_strategy.py:263-347), in theboss's order: the
 * mode that receives the approximated particles (randint(0, approximated_modes)),
 * the surviving particles of every occupied mode when `lossy` (the module's
 * choice(): one random() and a scan of loss_weights row `occupation`;
 * loss_weights is (max_occupation + 1)^2), approximated_modes phase uniforms,
 * then the C&C-B steps.  Outputs as in boss_bobs_uniform_predraw (no permutations).
 */
BOSS_API int boss_bobs_nonuniform_predraw(uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t m,
                                          const int32_t* base_state, int32_t approximated_modes,
                                          int32_t approximated_particles, const double* loss_weights,
                                          int32_t max_occupation, int32_t lossy, int32_t stride,
                                          int32_t* input_states, double* phase_uniforms, int32_t* randint_results,
                                          double* uniforms);

#ifdef __cplusplus
}
#endif

#endif /* BOSS_GB300_H */
