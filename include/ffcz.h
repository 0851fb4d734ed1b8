/*
 * ffcz.h -- C ABI of the GB300 (sm_103a) FFCz corrector and edit encoder.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (FFCZ_OK == 0, negative on failure).  The message of
 * the last failure on the calling thread is available from
 * ffcz_last_error().  Nothing here prints or exits the process; the C++
 * drop-in headers (projection_algorithm.cuh, HuffmanZSTDCoder.cuh) turn the
 * status codes back into the reference's behaviour (print + exit(1) for CUDA
 * errors, std::runtime_error for usage errors).
 *
 * Reference interface replaced by each group is cited as file:line of the
 * FFCz sources (projection_algorithm.cuh, projection_algorithm_impl.cuh,
 * projection_algorithm.cu, HuffmanZSTDCoder.cuh, fileIO.h).
 *
 * Array layouts (identical to the reference):
 *   spatial arrays   : Nx*Ny*Nz values of T, C order, z fastest.
 *   spectrum index k : (ix*Ny + iy)*(Nz/2+1) + kz, the unnormalised R2C
 *                      half spectrum of cufftPlan3d(Nx,Ny,Nz).
 *   frequency edits  : planar, 2*H values of T: [Re(0..H-1) | Im(0..H-1)],
 *                      H = Nx*Ny*(Nz/2+1).
 *   flag packs       : LSB-first bit i of byte b = flag of element 8b+i.
 *   Huffman streams  : MSB-first bitstream, zero padded to whole bytes.
 */
#ifndef FFCZ_H
#define FFCZ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FFCZ_OK                   0
#define FFCZ_ERR_INVALID         -1  /* bad argument / usage error            */
#define FFCZ_ERR_CUDA            -2  /* a CUDA runtime call failed            */
#define FFCZ_ERR_UNSUPPORTED     -3  /* size or mode not supported            */
#define FFCZ_ERR_NOT_INITIALIZED -4  /* solve before initialize (impl:822)    */
#define FFCZ_ERR_ZSTD            -5  /* libzstd missing or ZSTD error         */
#define FFCZ_ERR_CAPACITY        -6  /* caller buffer too small               */
#define FFCZ_ERR_CODE_TOO_LONG   -7  /* Huffman code longer than 32 bits      */
#define FFCZ_ERR_EMPTY           -8  /* empty input (HuffmanZSTDCoder:250)    */
#define FFCZ_ERR_IO              -9  /* file I/O failure (fileIO.cpp)         */

/* ---- element types ----------------------------------------------------- */
#define FFCZ_F32 0
#define FFCZ_F64 1

/* ---- flag-pack modes ---------------------------------------------------- */
/* Correct LSB-first packing of every flag (default). */
#define FFCZ_PACK_CORRECT   0
/* Reproduces projection_algorithm.cu:382-405 as launched by
 * projection_algorithm_impl.cuh:429-449: only the first ceil(nbytes/8) bytes
 * are written and they hold flags [0, nbytes); the remaining bytes, which the
 * reference leaves uninitialised, are zero. */
#define FFCZ_PACK_REFERENCE 1

/* ---- loop drivers --------------------------------------------------------- */
/* Whole iteration loop inside one CUDA graph with a device-side WHILE node. */
#define FFCZ_LOOP_GRAPH 0
/* Host-driven loop, one 8-byte device->host read per iteration (the
 * reference's structure, impl:835-852).  Same kernels, same results. */
#define FFCZ_LOOP_HOST  1

const char *ffcz_last_error(void);
const char *ffcz_version(void);

/* ======================================================================== *
 * Solver (replaces template<class T> class ProjectionSolver,               *
 * projection_algorithm.cuh:238-333, implemented in                        *
 * projection_algorithm_impl.cuh:1-910)                                     *
 * ======================================================================== */
typedef struct ffcz_solver ffcz_solver;

/* ProjectionSolver(Nx,Ny,Nz) -- impl:4-18 (allocation impl:27-61, plans
 * impl:109-122, accumulators zeroed impl:133-147). dtype = FFCZ_F32/F64. */
int ffcz_solver_create(size_t nx, size_t ny, size_t nz, int dtype,
                       ffcz_solver **out);
/* ~ProjectionSolver -- impl:20-25. NULL is accepted. */
int ffcz_solver_destroy(ffcz_solver *s);
/* Stream the solver launches on (cudaStream_t as void*; NULL = legacy
 * default stream, like the reference). */
int ffcz_solver_set_stream(ffcz_solver *s, void *stream);
/* FFCZ_LOOP_GRAPH (default) or FFCZ_LOOP_HOST. */
int ffcz_solver_set_loop_driver(ffcz_solver *s, int driver);
/* FFCZ_PACK_CORRECT (default) or FFCZ_PACK_REFERENCE. */
int ffcz_solver_set_pack_mode(ffcz_solver *s, int mode);
/* Iteration form of the all-abs loop (no counterpart in the reference,
 * whose iteration is cuFFT R2C + clamp kernel + cuFFT C2R + normalise,
 * projection_algorithm_impl.cuh:201-249):
 *   FFCZ_FORM_FUSED (default): five HBM passes per 3D iteration -- z R2C
 *     (spatial-clamp prologue), y forward, x forward + frequency clamp + x
 *     inverse in one pass, y inverse, z C2R (normalisation, violation);
 *   FFCZ_FORM_PLAIN: six -- the x forward pass stores the clamped spectrum
 *     and the x inverse is a pass of its own (2D: the same on y).
 * Both compute the reference's iteration; results agree to FP32 rounding
 * (the passes' stage lists differ).  Other constraint modes always run the
 * fused form.  FFCZ_ERR_UNSUPPORTED where no forward-with-clamp kernel
 * exists (float-float FP64 passes). */
#define FFCZ_FORM_FUSED 0
#define FFCZ_FORM_PLAIN 1
int ffcz_solver_set_form(ffcz_solver *s, int form);
/* Arithmetic of the radix-16 stages of the FP32 strided passes of length
 * 256 and 512 (no counterpart in the reference, which calls cuFFT):
 *   FFCZ_DFT_SIMT (default): register butterflies on the FP32 pipes;
 *   FFCZ_DFT_TENSOR: each radix-16 stage as 16-point DFT matrix products on
 *     the tensor cores (mma.sync m16n8k8, operands split into two TF32
 *     terms, three products, FP32 accumulation: ~21-bit products), the tile
 *     staged in shared memory; applies to the all-abs passes and forward
 *     transforms of those axes (the other axes and modes keep SIMT).
 * FFCZ_ERR_UNSUPPORTED for FP64 solvers or without such an axis. */
#define FFCZ_DFT_SIMT 0
#define FFCZ_DFT_TENSOR 1
int ffcz_solver_set_dft_stages(ffcz_solver *s, int stages);

/* How the FP32 strided (y, x) passes of compile-time lengths get their tiles
 * (no counterpart in the reference):
 *   FFCZ_STAGING_REGISTERS: each block loads its tile straight into
 *     registers (one tile per block, nothing in flight while it computes);
 *   FFCZ_STAGING_TMA: persistent blocks whose next tiles arrive in shared
 *     memory by tensor-map (TMA) copies issued ahead while the current tile
 *     is transformed; same arithmetic in the same order, identical results;
 *   FFCZ_STAGING_AUTO (default): registers until ffcz_solver_autotune,
 *     which times both per axis and keeps the faster.
 * FFCZ_ERR_UNSUPPORTED for TMA when no strided axis has a staged kernel
 * (FP64 solvers, lengths without compile-time kernels).  A staged pass that
 * waits about two seconds for a tile without it arriving gives up, and the
 * solve returns FFCZ_ERR_CUDA. */
/* When a solve compacts its edit accumulators (no counterpart in the
 * reference, whose solve_all_abs always extracts at its end, impl:850-852):
 *   FFCZ_EXTRACT_EAGER (default): at the end of every solve, as the reference;
 *   FFCZ_EXTRACT_ON_DEMAND: the solve leaves the compaction pending and the
 *     first call that reads its results (counts, min/max, streams, packs,
 *     device arrays, encode) or changes the edit arrays (reset, set,
 *     decode, autotune) runs it first.  Every call returns what it returns
 *     in the eager mode; a solve followed by ffcz_strict_finish then
 *     compacts once instead of twice.  A pending compaction runs before
 *     the mode changes. */
#define FFCZ_EXTRACT_EAGER 0
#define FFCZ_EXTRACT_ON_DEMAND 1
int ffcz_solver_set_extraction(ffcz_solver *s, int mode);

#define FFCZ_STAGING_REGISTERS 0
#define FFCZ_STAGING_TMA 1
#define FFCZ_STAGING_AUTO 2
int ffcz_solver_set_staging(ffcz_solver *s, int staging);
/* Tile choices of the solver: choice[3] (may be NULL) receives, per pass
 * (z, y, x), the tile variant (bit 0) and whether the pass runs TMA-staged
 * (bit 1); ms10 (may be NULL) the autotuner's last timings: (default,
 * alternative) ms of z, y and x with register staging, then (default,
 * alternative) ms of y and x TMA-staged; 0 where not timed. */
int ffcz_solver_get_tuning(ffcz_solver *s, int *choice, double *ms10);

/* initialize_all_abs(h_orig, eps, delta) -- impl:639-668.  x is a host
 * array of Nx*Ny*Nz elements of the solver's dtype; eps and delta are
 * converted to the solver's dtype. */
int ffcz_init_all_abs(ffcz_solver *s, const void *h_orig, double eps,
                      double delta);
/* Same, x already resident on the device. */
int ffcz_init_all_abs_device(ffcz_solver *s, const void *d_orig, double eps,
                             double delta);

/* solve_all_abs(h_err, max_iter, tol) -- impl:816-858: copies the initial
 * error e0 = x' - x from the host, runs the alternating projections and the
 * compaction (extract_compact_representation, impl:371-456).  tol is
 * converted to the solver's dtype. Does not print. */
int ffcz_solve_all_abs(ffcz_solver *s, const void *h_err, int max_iter,
                       double tol);
/* Same, e0 resident on the device (d_err is read, not modified). */
int ffcz_solve_all_abs_device(ffcz_solver *s, const void *d_err,
                              int max_iter, double tol);
/* Device-resident pair: e0 = x' - x is formed inside the first forward
 * pass (the subtraction projection_example.cu:173-176 does on the host).
 * d_orig must be the array given to the initialiser; it is not re-read. */
int ffcz_solve_all_abs_pair_device(ffcz_solver *s, const void *d_orig,
                                   const void *d_decomp, int max_iter,
                                   double tol);
/* ---- the other constraint modes (impl:598-637, 670-738, 772-814,
 * 860-902; kernels projection_algorithm.cu:93-145, 191-333) ---------------- */
#define FFCZ_MODE_ALL_ABS     0  /* every coefficient within +-delta       */
#define FFCZ_MODE_DIRECT      1  /* listed coefficients within +-delta_k   */
#define FFCZ_MODE_ALL_PTW     2  /* pointwise power-spectrum box, all k    */
#define FFCZ_MODE_PARTIAL_PTW 3  /* the same on listed coefficients        */
/* initialize(h_orig, h_freq_indices, h_delta_k, eps, num) -- impl:598-637.
 * h_delta_k: num values of the solver's dtype.  Indices must be < H; an
 * index listed twice keeps its smaller bound (the reference races there). */
int ffcz_init_direct(ffcz_solver *s, const void *h_orig,
                     const size_t *h_freq_indices, const void *h_delta_k,
                     double eps, size_t num_constraints);
/* initialize_all_ptw(h_orig, eps, delta_ptw) -- impl:670-697: also the
 * spectrum of x the pointwise box compares against. */
int ffcz_init_all_ptw(ffcz_solver *s, const void *h_orig, double eps,
                      double delta_ptw);
int ffcz_init_all_ptw_device(ffcz_solver *s, const void *d_orig, double eps,
                             double delta_ptw);
/* initialize_partial_ptw(h_orig, h_freq_indices, delta_ptw, eps, num) --
 * impl:699-738.  As in projection_algorithm.cu:276-289, constraint 0 is the
 * DC rule whatever index it lists; constraints 1.. get the pointwise box. */
int ffcz_init_partial_ptw(ffcz_solver *s, const void *h_orig,
                          const size_t *h_freq_indices, double delta_ptw,
                          double eps, size_t num_constraints);
/* solve(h_err, max_iter, tol) -- impl:772-814: the direct mode, or the
 * partial pointwise mode when initialize_partial_ptw ran last of the two
 * (the reference's solve() reads the direct mode's bounds in that case,
 * which initialize_partial_ptw never sets). */
int ffcz_solve(ffcz_solver *s, const void *h_err, int max_iter, double tol);
/* solve_all_ptw(h_err, max_iter, tol) -- impl:860-902. */
int ffcz_solve_all_ptw(ffcz_solver *s, const void *h_err, int max_iter,
                       double tol);
/* Any mode with e0 resident on the device (FFCZ_ERR_NOT_INITIALIZED when
 * the mode's initialiser did not run). */
int ffcz_solve_mode_device(ffcz_solver *s, int mode, const void *d_err,
                           int max_iter, double tol);

/* Projection loop only, without the compaction (impl:835-852). */
int ffcz_project_all_abs_device(ffcz_solver *s, const void *d_err,
                                int max_iter, double tol);
/* extract_compact_representation() -- impl:371-456 (flags, whole-array
 * min/max, scan, compaction, uint16 quantisation, flag packs). */
int ffcz_extract(ffcz_solver *s);
/* reset_edit_accumulators() -- impl:133-147.  Both accumulators are all
 * zeros afterwards; one nothing has written since its last clear is not
 * rewritten. */
int ffcz_reset_edit_accumulators(ffcz_solver *s);
/* Loads host arrays into the edit accumulators (2H planar frequency edits,
 * N spatial edits; either may be NULL to keep that accumulator), so that
 * ffcz_extract / ffcz_solver_encode compact and code edits produced
 * elsewhere.  The reference keeps its accumulators private
 * (projection_algorithm.cuh:77-78); this stands in for a caller writing
 * results_.d_freq_edits / d_spatial_edits before
 * extract_compact_representation (impl:371-456). */
int ffcz_set_edit_accumulators(ffcz_solver *s, const void *h_freq_edits,
                               const void *h_spatial_edits);
/* Waits for the solver's stream. */
int ffcz_solver_synchronize(ffcz_solver *s);

/* ---- results (impl:458-595, 904-910) ------------------------------------ */
/* iterations (impl:843), last convergence metric (impl:842) as double. */
int ffcz_get_iterations(ffcz_solver *s, int *iterations);
int ffcz_get_convergence(ffcz_solver *s, double *metric);
/* h_num_active_freq / h_num_active_spatial (impl:412, 424). */
int ffcz_get_active_counts(ffcz_solver *s, size_t *n_freq, size_t *n_spatial);
/* get_min/max_freq/spatial_edit (impl:573-595); values as double. */
int ffcz_get_minmax(ffcz_solver *s, double *fmin, double *fmax,
                    double *smin, double *smax);
/* get_results(h_err) -- impl:904-910: the corrected error e (x^ = x + e). */
int ffcz_get_results(ffcz_solver *s, void *h_err);
/* get_freq_edits_full / get_spatial_edits_full -- impl:555-571. */
int ffcz_get_freq_edits_full(ffcz_solver *s, void *dst, size_t cap_elems);
int ffcz_get_spatial_edits_full(ffcz_solver *s, void *dst, size_t cap_elems);
/* get_active_*_quant_edit_distances -- impl:507-529 (uint16). */
int ffcz_get_freq_quant(ffcz_solver *s, uint16_t *dst, size_t cap,
                        size_t *len);
int ffcz_get_spatial_quant(ffcz_solver *s, uint16_t *dst, size_t cap,
                           size_t *len);
/* get_active_*_edit_distances -- impl:531-553 (T). */
int ffcz_get_freq_compact(ffcz_solver *s, void *dst, size_t cap, size_t *len);
int ffcz_get_spatial_compact(ffcz_solver *s, void *dst, size_t cap,
                             size_t *len);
/* get_*_flags_pack -- impl:487-505; length is ceil(n/8) bytes. */
int ffcz_get_freq_flags_pack(ffcz_solver *s, uint8_t *dst, size_t cap,
                             size_t *len);
int ffcz_get_spatial_flags_pack(ffcz_solver *s, uint8_t *dst, size_t cap,
                                size_t *len);
/* get_freq_flags / get_spatial_flags -- impl:459-485, one byte per flag. */
int ffcz_get_freq_flags(ffcz_solver *s, uint8_t *dst, size_t cap,
                        size_t *len);
int ffcz_get_spatial_flags(ffcz_solver *s, uint8_t *dst, size_t cap,
                           size_t *len);
/* Device pointers of the solver-owned arrays (for zero-copy callers):
 * which = 0 e, 1 freq_edits, 2 spatial_edits, 3 freq quant, 4 spatial
 * quant, 5 freq pack, 6 spatial pack, 7 freq compact, 8 spatial compact,
 * 9 spectrum of x of the pointwise modes (Nx*Ny rows of pitch Hzp complex
 * values, Hzp = Nz/2+1 rounded up to 128 bytes; 0 bytes before an
 * initialize_*_ptw).  Read-only for callers: the solver knows when the
 * frequency-edit accumulator is still all zeros (nothing clamped since
 * ffcz_reset_edit_accumulators) and then compacts it without reading it. */
int ffcz_get_device_array(ffcz_solver *s, int which, void **dptr,
                          size_t *bytes);
/* Autotuner (no counterpart in the reference): times the default and an
 * alternative tile width of each pass that has compile-time kernels (z pair,
 * y pair, fused pass; reps launches each, on the solver's buffers) and keeps
 * the faster.  Results are unchanged (same arithmetic, same order); the edit
 * accumulators are cleared.  ms6 (may be NULL) receives the (default,
 * alternative) ms of z, y and x, 0 where a pass has no alternative. */
int ffcz_solver_autotune(ffcz_solver *s, int reps, double *ms6);
/* Arithmetic of an FP64 solver's pass kernels (an addition; the reference
 * computes in cuFFT double).  FFCZ_PRECISION_NATIVE (default): FP64.
 * FFCZ_PRECISION_SPLIT: the compile-time pass kernels of the power-of-two
 * lengths 128..512 keep FP64 in memory but compute in float-float (pairs of
 * FP32 values, ~48-bit significand, relative rounding ~1e-14 per operation)
 * on the FP32 pipes; other lengths stay FP64; the frequency and spatial
 * boxes and the violation are evaluated in FP64 (FP32 pre-checks skip the
 * values far inside them); ffcz_verify_bounds and ffcz_strict_finish keep
 * checking in FP64.  About 2x faster than native at 512^3.  Reselects the kernels (the
 * autotuner's choice is reset).  FP32 solvers accept NATIVE only. */
#define FFCZ_PRECISION_NATIVE 0
#define FFCZ_PRECISION_SPLIT  1
int ffcz_solver_set_precision(ffcz_solver *s, int precision);
/* FP64 check of the last solve's corrected error e on the device (no
 * counterpart in the reference): e widened exactly to FP64, its R2C in FP64
 * by an FP64 twin of the solver (created on first use), and
 *   spatial_max = max_i |e_i|,  freq_max = max_k max(|Re E_k|, |Im E_k|)
 * over the half spectrum.  The all-abs bounds hold when spatial_max <= eps
 * (+ the loop's tol) and freq_max <= delta. */
int ffcz_verify_bounds(ffcz_solver *s, double *spatial_max, double *freq_max);
/* Strict bounds (an addition; the reference stops once the spatial
 * violation is below tol, impl:845-848, so its e may exceed eps by up to tol
 * and meets delta only up to the FFT's rounding).  After an all-abs solve:
 *   1. e is clamped to E_T, the largest value of the solver's type <= eps
 *      (clamps recorded in the spatial edits);
 *   2. the certificate of ffcz_certify_bounds (the solver's own transform
 *      and a bound on its rounding) decides both bounds unless a
 *      coefficient comes within that bound of delta; then both bounds are
 *      checked in FP64 (ffcz_verify_bounds);
 *   3. while some |Re/Im F(e)_k| > delta, the loop runs again from the
 *      current e (max_iter, tol) on a frequency box shrunk by twice the worst
 *      overshoot (frequency edits accumulate as usual), then 1-2 again; at
 *      most max_rounds times.
 * Afterwards the iteration count is the total, and the compaction is redone
 * when the solve had extracted.  *met = 1 when spatial_max <= eps and
 * freq_max <= delta in FP64, eps and delta as the solver holds them (rounded
 * to its type at initialisation).  Any out pointer may be NULL. */
int ffcz_strict_finish(ffcz_solver *s, int max_iter, double tol, int max_rounds, int *rounds, int *met,
                       double *spatial_max, double *freq_max);
/* Certificate of both bounds without an FP64 transform (an addition): the
 * forward transform of e in the solver's own precision, max |Re/Im| over
 * the half spectrum (freq_max), and an a-posteriori bound on that
 * transform's rounding error (bound = 16 u L sqrt(N sum e_i^2), L = sum of
 * ceil(log2 n) over the axes + 2, u the unit roundoff of the passes; from
 * the FFT error analysis of Higham, Accuracy and Stability of Numerical
 * Algorithms, Thm 24.2, with 2.4x its constant).  *certified = 1 when
 * spatial_max <= eps and freq_max + bound <= delta: then both bounds hold
 * in exact arithmetic.  e and the accumulators are not changed; the
 * spectrum buffer is (a later ffcz_extract recomputes the compaction). */
int ffcz_certify_bounds(ffcz_solver *s, double *spatial_max, double *freq_max, double *bound, int *certified);
/* How the last ffcz_strict_finish decided: *certified = 1 when the
 * certificate did (no FP64 transform ran), with its freq_max and bound. */
int ffcz_get_strict_report(ffcz_solver *s, int *certified, double *freq_max, double *bound);
/* The spectrum of x of the pointwise modes (d_orig_freq, impl:612-623):
 * H interleaved complex values of the solver's dtype. */
int ffcz_get_orig_spectrum(ffcz_solver *s, void *h_dst, size_t cap_complex);
/* Sizes: n = Nx*Ny*Nz, h = Nx*Ny*(Nz/2+1). */
int ffcz_get_sizes(ffcz_solver *s, size_t *n, size_t *h);
/* Kernel launches issued since the last solve started (projection loop,
 * compaction, strict finish and FP64 checks, and any encode of its
 * streams). */
int ffcz_get_launch_count(ffcz_solver *s, long long *launches);
/* Per-pass timing: when on, CUDA events are recorded around each pass of
 * the first iteration of every solve (inside the captured graph).
 * ffcz_get_pass_times returns, for the last solve, each pass's elapsed ms
 * and its algorithmic bytes (one read + one write of the data it maps):
 * order z-forward, [y-forward], fused axis or clamp, [y-inverse],
 * z-inverse. */
int ffcz_solver_set_profiling(ffcz_solver *s, int on);
int ffcz_get_pass_times(ffcz_solver *s, double *ms, double *bytes, int cap,
                        int *npass);

/* ======================================================================== *
 * Batched form: many fields of uneven shapes in one graph launch           *
 * ======================================================================== */
/* No counterpart in the reference, whose CLI corrects one field per process
 * (projection_example.cu:160-246).  A batch groups solver handles, each
 * created for its own field shape and initialised (ffcz_init_all_abs*) with
 * its own eps and delta.  ffcz_batch_solve_pair_device runs, for every
 * field at once, what ffcz_solve_all_abs_pair_device runs for one: the
 * projection loop of each field is a device-side while loop of its own
 * inside one CUDA graph, so a field retires when it converges (or reaches
 * max_iter) while the others keep iterating, and its compaction follows in
 * the same graph.  Each field's results equal those of
 * ffcz_solve_all_abs_pair_device on its own handle, bit for bit, and are
 * read through that handle's getters and ffcz_solver_encode.
 *   solvers : nfields distinct handles on the current device; the batch
 *             keeps the pointers (destroy the batch before them).
 *   d_orig[f], d_decomp[f] : device arrays of field f (16-byte aligned).
 * The call runs on the batch's stream (ffcz_batch_set_stream; legacy
 * default stream otherwise) and returns after it finished.  A graph is
 * built on the first call with a set of arguments; the two most recent sets
 * keep theirs, so inputs that alternate between two buffer sets (the next
 * step's fields copied in while this step runs) capture nothing new. */
typedef struct ffcz_batch ffcz_batch;
int ffcz_batch_create(ffcz_solver *const *solvers, int nfields,
                      ffcz_batch **out);
int ffcz_batch_destroy(ffcz_batch *b);
int ffcz_batch_set_stream(ffcz_batch *b, void *stream);
/* ffcz_reset_edit_accumulators of every field, on the batch's stream, with
 * one synchronisation. */
int ffcz_batch_reset_edit_accumulators(ffcz_batch *b);
int ffcz_batch_solve_pair_device(ffcz_batch *b, const void *const *d_orig,
                                 const void *const *d_decomp, int max_iter,
                                 double tol);

/* ======================================================================== *
 * Huffman + ZSTD coder (replaces SimpleCudaHuffmanZstdCompressor<T>,       *
 * HuffmanZSTDCoder.cuh:236-451, cudaHuffmanZstdCompress/Decompress :454-470)*
 * ======================================================================== */
typedef struct ffcz_huff_result ffcz_huff_result;

/* ZSTD framing of the Huffman bitstream. */
#define FFCZ_ZSTD_SINGLE 0   /* one ZSTD_compress call (reference :359-375) */
#define FFCZ_ZSTD_CHUNKED 1  /* independent frames over host threads; the  */
                             /* concatenation decodes with ZSTD_decompress */
#define FFCZ_ZSTD_NONE 2     /* Huffman bitstream only (no ZSTD stage)     */

/* compress(data, level) for T = uint16_t / uint8_t from HOST data --
 * HuffmanZSTDCoder.cuh:248-376.  Histogram, code lengths, bit offsets and
 * bit packing run on the GPU; the codebook (:85-178) and ZSTD on the host. */
int ffcz_huff_compress_u16(const uint16_t *h_data, size_t n, int zstd_level,
                           ffcz_huff_result **out);
int ffcz_huff_compress_u8(const uint8_t *h_data, size_t n, int zstd_level,
                          ffcz_huff_result **out);
/* Same from DEVICE data, with the ZSTD framing mode and a stream. */
int ffcz_huff_compress_device(const void *d_data, size_t n, int symbol_bytes,
                              int zstd_level, int zstd_mode, void *stream,
                              ffcz_huff_result **out);
void ffcz_huff_result_free(ffcz_huff_result *r);
/* Symbol histogram of n device-resident symbols (1 or 2 bytes each,
 * 16-byte aligned) into h_hist (256 or 65536 counts), computed on the GPU
 * with the encoder's shared-memory histogram on `stream`; the work of
 * cudaFrequencyCount (HuffmanZSTDCoder.cuh:48-83) before its compaction to
 * ascending (symbol, count) pairs. */
int ffcz_huff_histogram_device(const void *d_data, size_t n, int symbol_bytes, void *stream,
                               uint32_t *h_hist);
/* The Huffman tree of buildHuffmanTree (HuffmanZSTDCoder.cuh:85-152) for n
 * leaves of weights freqs[0..n-1] (the ascending symbols' counts): 2n-1
 * nodes, leaves first, internal nodes in merge order, each merging the two
 * smallest (weight, node index) pairs with the first as its left (0)
 * child; -1 for no child.  *root = 2n-2 (0 for one leaf, -1 for none). */
int ffcz_huff_tree(const uint32_t *freqs, size_t n, int32_t *left, int32_t *right, uint64_t *weights,
                   int32_t *root);
/* The code table the encoder builds from a dense histogram (nbins counts,
 * host memory, no GPU): cudaFrequencyCount's ascending (symbol, count)
 * pairs, buildHuffmanTree and generateCodesRecursive
 * (HuffmanZSTDCoder.cuh:48-178): symbols with a non-zero count in
 * ascending order, their codes (MSB-first, the low 32 bits) and lengths
 * (one symbol: code 0, length 1).  *n receives the number of symbols;
 * FFCZ_ERR_CAPACITY when it exceeds cap. */
int ffcz_huff_codebook(const uint32_t *hist, size_t nbins, uint32_t *symbols, uint32_t *codes, int32_t *lengths,
                       size_t cap, size_t *n);
/* CompressionResult fields (:240-246). */
int ffcz_huff_result_sizes(const ffcz_huff_result *r, size_t *compressed_bytes,
                           size_t *bitstream_bytes, size_t *num_elements,
                           size_t *num_symbols);
int ffcz_huff_result_compressed(const ffcz_huff_result *r, uint8_t *dst,
                                size_t cap);
/* The uncompressed Huffman bitstream (before ZSTD). */
int ffcz_huff_result_bitstream(const ffcz_huff_result *r, uint8_t *dst,
                               size_t cap);
/* Code table as three parallel arrays in ascending symbol order. */
int ffcz_huff_result_codes(const ffcz_huff_result *r, uint32_t *symbols,
                           uint32_t *codes, int32_t *lengths, size_t cap);
/* Read-only view of a result's buffers, valid until the result is freed:
 * which = 0 compressed bytes, 1 bitstream bytes, 2 symbols (uint32),
 * 3 codes (uint32), 4 lengths (int32); *count = elements. */
int ffcz_huff_result_view(const ffcz_huff_result *r, int which,
                          const void **ptr, size_t *count);

/* The ZSTD stage alone (HuffmanZSTDCoder.cuh:359-375) on host bytes, so
 * that callers can run it on their own threads, overlapped with the GPU
 * work of later fields.  FFCZ_ZSTD_SINGLE gives exactly ZSTD_compress's
 * bytes.  ffcz_zstd_bound is an upper bound on the output size. */
size_t ffcz_zstd_bound(size_t n);
int ffcz_zstd_compress(const uint8_t *src, size_t n, int level, int mode,
                       uint8_t *dst, size_t cap, size_t *out_len);

/* decompress(...) -- HuffmanZSTDCoder.cuh:378-450: ZSTD_decompress, then a
 * prefix decode with the same stop and bit-skip rules.  out must hold
 * num_elements symbols; *out_len receives the decoded count. */
int ffcz_huff_decompress_u16(const uint8_t *comp, size_t comp_len,
                             const uint32_t *symbols, const uint32_t *codes,
                             const int32_t *lengths, size_t num_symbols,
                             size_t num_elements, size_t bitstream_bytes,
                             uint16_t *out, size_t *out_len);
int ffcz_huff_decompress_u8(const uint8_t *comp, size_t comp_len,
                            const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols,
                            size_t num_elements, size_t bitstream_bytes,
                            uint8_t *out, size_t *out_len);

/* Encode the solver's four streams the way projection_example.cu:230-246
 * does (frequency quantised edits, frequency flag pack, spatial quantised
 * edits, spatial flag pack; a pair only when its count is non-zero).
 * out[4] receives results or NULL for skipped streams; the caller frees. */
int ffcz_solver_encode(ffcz_solver *s, int zstd_level, int zstd_mode,
                       ffcz_huff_result **out4);

/* ======================================================================== *
 * Decoder side (no counterpart in the reference beyond the host decode of  *
 * HuffmanZSTDCoder.cuh:378-450 and the commented-out reconstruction of     *
 * projection_algorithm_impl.cuh:912-985)                                   *
 * ======================================================================== */
/* GPU prefix decode of a Huffman bitstream with the rules of the host
 * decoder above (same output, symbol for symbol): d_bits is DEVICE memory of
 * nbytes; up to num_elements symbols (symbol_bytes 1 or 2) go to d_out
 * (device); *decoded receives the count.  Runs on `stream`, returns after
 * it finished. */
int ffcz_huff_decode_device(const uint8_t *d_bits, size_t nbytes,
                            const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols,
                            size_t num_elements, int symbol_bytes, void *d_out,
                            size_t *decoded, void *stream);
/* ZSTD_decompress on the host, then the GPU decode into d_out (device). */
int ffcz_huff_zstd_decompress_device(const uint8_t *comp, size_t comp_len,
                                     const uint32_t *symbols,
                                     const uint32_t *codes,
                                     const int32_t *lengths,
                                     size_t num_symbols, size_t num_elements,
                                     size_t bitstream_bytes, int symbol_bytes,
                                     void *d_out, size_t *decoded,
                                     void *stream);
/* A coder result rebuilt from its stored parts (ZSTD frame, code table,
 * counts) for decoding.  bitstream: the Huffman bitstream when at hand;
 * NULL: recovered here from `compressed` (ZSTD_decompress into
 * bitstream_bytes bytes). */
int ffcz_huff_result_create(const uint8_t *compressed, size_t comp_len,
                            const uint8_t *bitstream, size_t bitstream_bytes,
                            const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols,
                            size_t num_elements, ffcz_huff_result **out);
/* Reconstruction of the corrected field from decoded edit streams:
 *   x^ = x' + (C2R(F)/N + S)
 * F = the frequency edits (planar Re | Im over the half spectrum), S = the
 * spatial edits, each rebuilt from its flag pack (LSB-first, FFCZ_PACK_CORRECT
 * layout) and its uint16 codes dequantised as q/65535*(max-min)+min in T
 * (the inverse of projection_algorithm.cu:447-455, following :638).  All
 * arrays are device memory; d_decomp = x', d_out = x^ (N values of the
 * solver's dtype; may alias neither input).  Uses the solver's spectrum,
 * e and spatial-edit buffers (a previous solve's results are overwritten;
 * afterwards ffcz_get_spatial_edits_full returns the dequantised spatial
 * edits).  Returns after the solver's stream finished. */
int ffcz_reconstruct_device(ffcz_solver *s, const void *d_decomp,
                            const uint16_t *d_freq_quant, size_t n_freq,
                            const uint8_t *d_freq_pack, double freq_min,
                            double freq_max, const uint16_t *d_spatial_quant,
                            size_t n_spatial, const uint8_t *d_spatial_pack,
                            double spatial_min, double spatial_max,
                            void *d_out);
/* The whole decoder from the four coder results ffcz_solver_encode returns
 * (frequency codes, frequency flag pack, spatial codes, spatial flag pack;
 * NULL for an empty pair): GPU Huffman decode of each stream, then
 * ffcz_reconstruct_device.  min/max are ffcz_get_minmax's values. */
int ffcz_solver_decode(ffcz_solver *s, const void *d_decomp,
                       ffcz_huff_result *const *in4, double freq_min,
                       double freq_max, double spatial_min,
                       double spatial_max, void *d_out);

/* ---- base compressor ----------------------------------------------------- */
/* A uniform scalar quantiser producing x' on the GPU (the step before the
 * corrector; the reference reads x' from a file, projection_example.cu:
 * 160-176): q_i = rint(x_i / 2eps) (half to even), x'_i = T(2eps * q_i), in
 * FP64.  d_index (optional, n int32) receives q.  Returns after `stream`
 * finished. */
int ffcz_base_quantize_device(const void *d_x, size_t n, int dtype, double eps,
                              void *d_xprime, int32_t *d_index, void *stream);

/* ---- the .ffcz container ------------------------------------------------ */
/* The reference's CLI parses -z/-o but writes nothing (projection_example.cu:
 * 75-86, 255-256).  One file holds what the decoder needs besides x': shape,
 * dtype, bounds, min/max of both edit arrays and the four coder results
 * (each with its code table in writeMap's layout, fileIO.cpp:3-33).  Layout
 * in ffcz_gb300/csrc/container.cpp. */
typedef struct {
  uint32_t dtype;       /* FFCZ_F32 / FFCZ_F64 */
  uint32_t pack_mode;   /* flag-pack mode of the streams */
  uint64_t nx, ny, nz;
  double eps, delta;
  double freq_min, freq_max, spatial_min, spatial_max;
  uint32_t iterations;
} ffcz_container_header;
/* Header of the solver's last solve (shape, dtype, bounds, min/max,
 * iterations, pack mode). */
int ffcz_solver_container_header(ffcz_solver *s, ffcz_container_header *h);
/* in4: ffcz_solver_encode's four results (NULL = absent). */
int ffcz_container_write(const char *path, const ffcz_container_header *h,
                         ffcz_huff_result *const *in4);
/* Reads a container; out4 receives four new results (NULL = absent, caller
 * frees) with their bitstreams restored, ready for ffcz_solver_decode. */
int ffcz_container_read(const char *path, ffcz_container_header *h,
                        ffcz_huff_result **out4);

/* ======================================================================== *
 * Allocation-free compaction                                               *
 * ======================================================================== */
/* No counterpart in the reference.  The compaction of one edit accumulator
 * (what ffcz_extract does per array: flags |v| > 1e-7, whole-array min and
 * max, scatter of the active values, their uint16 codes and the flag pack)
 * for callers that cannot allocate device memory: applications that
 * reserve the GPU's memory up front in their own pool and forbid further
 * device allocations, and latency-bound pipelines that cannot afford the
 * implicit device synchronisation of cudaMalloc/cudaFree.  It calls no
 * allocator; its scratch is a fixed FFCZ_NOALLOC_SCRATCH_BYTES device array
 * inside the library, held by every GPU that loads it until process exit.
 *   d_edits   : n values of dtype (FFCZ_F32 / FFCZ_F64), device memory,
 *               16-byte aligned (read with 16-byte vector loads);
 *               n <= FFCZ_NOALLOC_MAX_ELEMS, else FFCZ_ERR_CAPACITY.
 *   d_compact : room for n values of dtype, aligned to the element size;
 *               receives the active values.
 *   d_quant   : room for n uint16, 2-byte aligned; receives their codes.
 *   d_pack    : 4-byte aligned, room for 4*ceil(n/32) bytes; receives the
 *               flag pack (FFCZ_PACK_CORRECT or FFCZ_PACK_REFERENCE).
 *   count, min_edit, max_edit : host outputs (min/max may be NULL).
 * A misaligned pointer returns FFCZ_ERR_INVALID before anything runs.
 * The call runs on `stream` and returns after it finished.  Every call
 * resolves the scratch array's device address on the current device (so
 * it stays right after cudaDeviceReset); the first call on a device may
 * load the library's device code, so make it before any stream capture.
 * All calls on a device share the scratch, so calls that overlap on the
 * GPU race. */
#define FFCZ_NOALLOC_MAX_ELEMS 67108864u      /* 16384 blocks of 4096 values */
#define FFCZ_NOALLOC_SCRATCH_BYTES 328192u
int ffcz_compact_quantize_noalloc(const void *d_edits, size_t n, int dtype,
                                  void *d_compact, uint16_t *d_quant,
                                  uint8_t *d_pack, int pack_mode,
                                  void *stream, size_t *count,
                                  double *min_edit, double *max_edit);

/* ======================================================================== *
 * File formats (fileIO.h:17-55, fileIO.cpp:3-85)                           *
 * ======================================================================== */
/* readRawArrayBinary -- fileIO.cpp:35-76: headerless array; the file size
 * must equal n*elem_bytes exactly. */
int ffcz_read_raw(const char *path, void *dst, size_t n, size_t elem_bytes);
/* writeRawArrayBinary / writeVectorBinary -- fileIO.h:23-55. */
int ffcz_write_raw(const char *path, const void *src, size_t n,
                   size_t elem_bytes);
/* writeMap / readMap -- fileIO.cpp:3-33: size_t n, then n x (int key,
 * uint32 code, int len), keys ascending. */
int ffcz_write_map(const char *path, const int32_t *keys,
                   const uint32_t *codes, const int32_t *lens, size_t n);
int ffcz_read_map(const char *path, int32_t *keys, uint32_t *codes,
                  int32_t *lens, size_t cap, size_t *n);

#ifdef __cplusplus
}
#endif
#endif /* FFCZ_H */
