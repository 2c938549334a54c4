/*
 * gw.h -- C ABI of the GB300 event-reweighting engine (libgw.so).
 *
 * This is the drop-in boundary for GUNDAM's Cache::Manager GPU path.  Every
 * entry point is `extern "C"`, takes plain pointers and sizes, and returns an
 * int status (GW_OK == 0).  No C++ exception crosses the boundary; the text of
 * the last failure is returned by gw_last_error().
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the GUNDAM source tree).  The reference drives its cache through
 * a per-type operator API filled by Cache::Manager::Update
 * (src/CacheManager/src/CacheManager.cpp:477-740) and evaluated by
 * Cache::Manager::Fill (src/CacheManager/src/CacheManager.cpp:750-810); the
 * same calls exist here with the same argument meaning.
 *
 * Semantics follow the reference's CPU propagation, which is the oracle:
 *   - norm dials are clamped like every other dial
 *     (src/DialDictionary/DialEngine/src/DialCollection.cpp:453-454);
 *   - the event-weight cap applies to the dial product before the base weight
 *     (src/DialDictionary/DialEngine/src/EventDialCache.cpp:156-171);
 *   - empty histogram bins sum to 0 (src/SamplesManager/src/Histogram.cpp:107-135);
 *   - parameter mirroring uses the fmod form
 *     (src/DialDictionary/DialEngine/src/DialInputBuffer.cpp:44-89).
 *
 * Threading: one host thread per engine at a time.  Calls on different engines
 * are independent.
 */
#ifndef GW_H
#define GW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  GW_OK = 0,
  GW_ERR_ARG = 1,            /* bad argument (index out of range, bad size) */
  GW_ERR_STATE = 2,          /* call not valid in the engine's current state */
  GW_ERR_CUDA = 3,           /* CUDA runtime error */
  GW_ERR_NOMEM = 4,          /* host or device allocation failed */
  GW_ERR_LIMIT = 5,          /* a layout limit was exceeded (see gw_last_error) */
  GW_ERR_DEVICE_TIMEOUT = 6, /* a bounded device-side wait gave up */
  GW_ERR_NOT_FINITE = 7      /* a non-finite table entry or parameter */
};

/* ---- dial types (one per Cache::Weight::* calculator) ------------------ */
enum {
  GW_DIAL_NORM = 1,      /* Cache::Weight::Normalization  (WeightNormalization.cpp:96-118) */
  GW_DIAL_MONOTONIC = 2, /* Cache::Weight::MonotonicSpline (WeightMonotonicSpline.cpp:286-321) */
  GW_DIAL_UNIFORM = 3,   /* Cache::Weight::UniformSpline  (WeightUniformSpline.cpp:276-326) */
  GW_DIAL_GENERAL = 4,   /* Cache::Weight::GeneralSpline  (WeightGeneralSpline.cpp:248-306) */
  GW_DIAL_COMPACT = 5,   /* Cache::Weight::CompactSpline  (WeightCompactSpline.cpp:252-288) */
  GW_DIAL_GRAPH = 6,     /* Cache::Weight::Graph          (WeightGraph.cpp:264-290) */
  GW_DIAL_BILINEAR = 7,  /* Cache::Weight::Bilinear       (WeightBilinear.cpp:152-181) */
  GW_DIAL_BICUBIC = 8,   /* Cache::Weight::Bicubic        (WeightBicubic.cpp:151-181) */
  GW_DIAL_TABULATED = 9, /* Cache::Weight::Tabulated      (WeightTabulated.cpp:134-150) */
  GW_DIAL_KRIGED = 10    /* Cache::Weight::Kriged         (WeightKriged.cpp:178-202) */
};

/* ---- precision of dial math and of the per-event weight product -------- */
enum {
  GW_FP64 = 0, /* everything in FP64, as the reference (WeightBase.h:19) */
  GW_FP32 = 1, /* dials + weight product in FP32; bin sums, sum of w^2, LLH in FP64 */
  GW_DF64 = 2  /* dials + weight product in double-float (two FP32 words per value, ~48
                  significant bits, on the FP32 pipe); bin sums, sum of w^2, LLH in FP64 */
};

/* ---- gw_config.flags: stored form of Catmull-Rom (monotonic, compact)
 * splines.  Knot values only, [low, 1/step, y x n], the reference's own data,
 * with the knot slopes formed in the kernel (fewer bytes per evaluation); or
 * with the slopes precomputed on the host, [low, 1/step, (y, slope) x n]
 * (less arithmetic per evaluation).  No flag: knot values for FP32 engines
 * with k_max == 1 (a bandwidth-bound evaluation), the grid form below for
 * engines with k_max >= 32 (their batched evaluation is bound by arithmetic
 * and instruction issue, not bytes) and for engines with 16 <= k_max < 32
 * whose grid table stays within 32 KB, else the coefficient form for FP64
 * engines with 16 <= k_max < 32; precomputed slopes otherwise.  Results agree
 * within the precision's rounding; in FP64
 * the per-event weights are identical (the bin sums then differ only in the
 * grouping of their FP64 partial sums, as the tiles are cut differently). */
enum {
  GW_FLAG_SPLINE_KNOTS = 1,
  GW_FLAG_SPLINE_SLOPES = 2,
  /* Monotonic, compact and uniform splines stored per interval as the
   * power-basis coefficients of the cubic the reference evaluates there,
   * [-low/step, 1/step, 0, 0, (c0, c1, c2, c3) x (n + 1)], with one interval
   * before the first knot and one after the last holding the reference's
   * extrapolation (for Catmull-Rom splines the end difference as the outer
   * slope): one 16-byte load and three multiply-adds per point, about 2.2x
   * the bytes of the slope form.  For batched evaluation, where the
   * arithmetic, not the bytes, bounds the kernel. */
  GW_FLAG_SPLINE_COEFS = 3,
  /* The coefficient form with the knot grid shared: monotonic, compact and
   * uniform splines whose (parameter, first knot, step, knot count) agree
   * share one grid (up to 16384 grids; splines of further grids keep the
   * coefficient form), their payload the coefficient blocks alone, and the
   * interval and fraction of each grid at each point are formed once per
   * evaluation, beside the parameter mirroring, instead of once per dial.
   * Per-event weights are identical to the coefficient form's. */
  GW_FLAG_SPLINE_GRID = 4
};

/* ---- likelihood evaluated after the histogram step --------------------- */
enum {
  GW_LLH_NONE = 0,
  GW_LLH_POISSON = 1,                /* PoissonLogLikelihood.h:19-53 */
  GW_LLH_BARLOW_BEESTON_OA2021 = 2   /* BarlowBeestonBanff2022.h:150-294 ("BarlowLLH_BANFF_OA2021") */
};

/* ---- device table functions (tables recomputed on the GPU) ------------- */
enum {
  /* T_j = 1 - a*sin^2(b*1.267/E_j + c)*(1 + d*(ln E_j - e))*f, parameters
   * (a,b,c,d,e,f) read from six fit parameters. */
  GW_TABLE_FN_OSCILLATION = 1
};

typedef struct gw_engine gw_engine;

/* Sizes fixed at construction.  Mirrors Cache::Manager::Build's counting pass
 * (CacheManager.cpp:198-475): results = cached events, params = cached
 * parameters, bins = histogram cells over all samples. */
typedef struct gw_config {
  int32_t n_results;  /* events in the cache */
  int32_t n_params;   /* parameters in the cache (<= 65535) */
  int32_t n_bins;     /* global histogram cells */
  int32_t k_max;      /* largest number of parameter points per gw_eval (>= 1) */
  int32_t precision;  /* GW_FP64, GW_FP32 or GW_DF64 */
  int32_t device;     /* CUDA device ordinal */
  int32_t tile_bytes; /* payload bytes per tile; 0 = default (FP32: 28672, 32768 with k_max >= 16;
                         FP64 and double-float: 40960) */
  int32_t flags;      /* 0 or one GW_FLAG_SPLINE_* value */
} gw_config;

/* ---- engine lifetime --------------------------------------------------- */

/* Cache::Manager::HasCUDA -> Cache::Parameters::UsingCUDA
 * (CacheManager.cpp:190-192; CacheParameters.cpp:12-18): writes 1 when the
 * library's kernels were compiled by the CUDA compiler (always, for libgw),
 * else 0.  Needs no device. */
int gw_using_cuda(int32_t* using_cuda);

/* Cache::Manager::HasGPU (CacheManager.h:78; CacheParameters.cpp:24-79).
 * Writes 1 when a usable CUDA device exists, else 0. */
int gw_has_gpu(int32_t* has_gpu);

/* new Cache::Manager(...) (CacheManager.cpp:46-188). */
int gw_create(const gw_config* config, gw_engine** engine);

/* Cache::Manager destructor. */
int gw_destroy(gw_engine* engine);

/* Copies the text of the last error on this engine (or, with engine == NULL,
 * the last gw_create failure of this thread) into buf. Replaces LogThrow. */
int gw_last_error(const gw_engine* engine, char* buf, size_t len);

/* ---- Cache::Parameters (CacheParameters.h:53-73) ----------------------- */
int gw_set_lower_mirror(gw_engine* e, int32_t par, double value); /* SetLowerMirror, CacheParameters.cpp:162-166 */
int gw_set_upper_mirror(gw_engine* e, int32_t par, double value); /* SetUpperMirror, CacheParameters.cpp:174-178 */
int gw_set_lower_clamp(gw_engine* e, int32_t par, double value);  /* SetLowerClamp,  CacheParameters.cpp:186-190 */
int gw_set_upper_clamp(gw_engine* e, int32_t par, double value);  /* SetUpperClamp,  CacheParameters.cpp:198-202 */
/* allowDialExtrapolation of the parameter's dials (DialCollection.h:200;
 * MonotonicSpline.cpp:78-81; Graph.cpp:48-51). Default: allowed. */
int gw_set_extrapolation(gw_engine* e, int32_t par, int32_t allow);

/* ---- Cache::Weights (CacheWeights.h:68-122) ---------------------------- */
int gw_set_initial_value(gw_engine* e, int32_t result, double value); /* SetInitialValue, CacheWeights.h:121 */
/* Batched form: values[i] for results [first, first+n). */
int gw_set_initial_values(gw_engine* e, int32_t first, int32_t n, const double* values);

/* ---- dial calculators (per-dial operator API) -------------------------- */
/* Normalization::ReserveNorm (WeightNormalization.h:65). */
int gw_reserve_norm(gw_engine* e, int32_t result, int32_t par);
/* {Monotonic,Uniform,General,Compact}Spline::AddSpline (WeightMonotonicSpline.h:113,
 * WeightUniformSpline.h:103, WeightGeneralSpline.h:104, WeightCompactSpline.h:113).
 * data is the dial's getDialData() vector:
 *   MONOTONIC, COMPACT: [low, step, y_0 .. y_{n-1}]
 *   UNIFORM:            [low, step, (y, dy/dx) x n]
 *   GENERAL:            [low, step, (y, dy/dx, x) x n] */
int gw_add_spline(gw_engine* e, int32_t type, int32_t result, int32_t par,
                  const double* data, int32_t n_data);
/* Graph::AddGraph (WeightGraph.h:89); data = [(y, x) x n]. */
int gw_add_graph(gw_engine* e, int32_t result, int32_t par, const double* data, int32_t n_data);
/* Bilinear::AddData / Bicubic::AddData (WeightBilinear.h:92, WeightBicubic.h:95);
 * data = [nx, ny, x[nx], y[ny], z[nx*ny]] with z row-major over x. */
int gw_add_surface(gw_engine* e, int32_t type, int32_t result, int32_t par1, int32_t par2,
                   const double* data, int32_t n_data);
/* Tabulated::AddData (WeightTabulated.h:57): v = f*T[index] + (1-f)*T[index+1]. */
int gw_add_tabulated(gw_engine* e, int32_t result, int32_t table, int32_t index, double fraction);
/* Kriged::AddData (WeightKriged.h:57): v = sum_j w_j * T[index_j]. */
int gw_add_kriged(gw_engine* e, int32_t result, int32_t table, int32_t n,
                  const int32_t* index, const float* weight);

/* Batched form of all of the above (no reference counterpart; one call per
 * block of dials).  Dial i has type[i], result[i], par0[i], par1[i] (-1 when
 * unused) and data[data_start[i] .. data_start[i+1]) in the formats above;
 * TABULATED data = [table, index, fraction], KRIGED data =
 * [table, m, index_0..index_{m-1}, weight_0..weight_{m-1}]. */
int gw_add_dials(gw_engine* e, int64_t n, const uint8_t* type, const int32_t* result,
                 const int32_t* par0, const int32_t* par1, const int64_t* data_start,
                 const double* data);

/* ---- tables for TABULATED / KRIGED dials ------------------------------- */
/* Registers a table of `size` entries (the std::vector<double>* a dial
 * borrows in WeightTabulated.h:57 / WeightKriged.h:57). */
int gw_create_table(gw_engine* e, int32_t size, int32_t* table);
/* Host refresh of a table (WeightTabulated.cpp:161-171, WeightKriged.cpp:213-223).
 * Takes effect at the next gw_eval. */
int gw_set_table(gw_engine* e, int32_t table, const double* values, int32_t size);
/* Response clamp of the table's dials (DialResponseSupervisor.cpp:10-18). */
int gw_set_table_clamp(gw_engine* e, int32_t table, double lower, double upper);
/* Recompute the table on the device from fit parameters at every point
 * (replaces the host updateTable plugin, KrigedDialFactory.cpp:135-145).
 * params[6] are fit-parameter indices, nodes[size] the energies E_j. */
int gw_set_table_function(gw_engine* e, int32_t table, int32_t fn, const int32_t* params,
                          int32_t n_params, const double* nodes, int32_t size);

/* ---- Cache::HistogramSum (CacheRecursiveSums.h:84-152) ------------------ */
int gw_set_event_index(gw_engine* e, int32_t result, int32_t bin);   /* SetEventIndex, CacheRecursiveSums.h:107 */
int gw_set_event_indices(gw_engine* e, int32_t first, int32_t n, const int32_t* bins);
int gw_set_maximum_event_weight(gw_engine* e, double maximum);        /* SetMaximumEventWeight, :111 */

/* ---- likelihood (JointProbabilityBase.h:37-54; LikelihoodInterface.cpp:165-215) */
int gw_set_data(gw_engine* e, const double* data, int32_t n_bins);
int gw_set_likelihood(gw_engine* e, int32_t llh_type);
/* Gaussian prior penalty (x-mean)^T inv_cov (x-mean) (LikelihoodInterface.cpp:186-215).
 * inv_cov is n_params*n_params row-major; NULL clears the prior. */
int gw_set_prior(gw_engine* e, const double* mean, const double* inv_cov);

/* Eigen-decomposed parameter set (ParameterSet::propagateEigenToOriginal,
 * ParameterSet.cpp:766-780; ParametersManager::convertEigenToOrig,
 * ParametersManager.cpp:329-334): parameters [first, first + n) passed to
 * gw_eval are eigen parameters, and the engine forms the original ones as
 * V * given (V [n x n] row-major, columns = eigenvectors) on the device before
 * mirroring and the dials.  The prior penalty applies to the parameters as
 * passed (the reference's eigen-mode penalty).  Blocks may not overlap. */
int gw_add_eigen_block(gw_engine* e, int32_t first, int32_t n, const double* V);

/* Packs, sorts, validates and uploads everything (RecursiveSums::Initialize,
 * CacheRecursiveSums.cpp:92-153, plus the hemi uploads).  After this the
 * builder calls above return GW_ERR_STATE. */
int gw_initialize(gw_engine* e);

/* ---- evaluation -------------------------------------------------------- */
/* Cache::Manager::Fill + CopyHistogramContents + the per-bin likelihood
 * (CacheManager.cpp:750-866; LikelihoodInterface.cpp:165-178), for K
 * parameter points at once.  Host buffers:
 *   params   [K * n_params]  parameter values (row k = point k)
 *   sums     [K * n_bins]    sum of weights per bin        (may be NULL)
 *   sums2    [K * n_bins]    sum of squared weights per bin (may be NULL)
 *   llh      [K]             stat + penalty                 (may be NULL)
 *   llh_stat [K]             stat part only                 (may be NULL)
 * Blocks until the results are on the host. */
int gw_eval(gw_engine* e, const double* params, int32_t K, double* sums, double* sums2,
            double* llh, double* llh_stat);

/* Same as gw_eval with DEVICE pointers, asynchronous on `stream`
 * (a cudaStream_t; NULL = the engine's own stream).  Any output may be NULL.
 * All evaluations of one engine share its scratch arrays, so the engine
 * orders them on the GPU: each call's launches wait for the previous call's,
 * whichever stream that used (gw_eval included), through an event recorded
 * at the end of every call.  While `stream` is being captured into the
 * caller's own CUDA graph no such wait or record is added; the caller then
 * orders the captured work against other calls on the engine itself. */
int gw_eval_device(gw_engine* e, const double* d_params, int32_t K, double* d_sums,
                   double* d_sums2, double* d_llh, double* d_llh_stat, void* stream);

/* Waits for the engine's outstanding work and reports device-side errors
 * (GW_ERR_DEVICE_TIMEOUT when a bounded wait gave up). */
int gw_sync(gw_engine* e);

/* Capture the K-point launch chain in a CUDA graph (on != 0) or go back to
 * plain launches. */
int gw_use_graph(gw_engine* e, int32_t on);

/* Times the batched kernel shapes for K points and keeps the fastest
 * (points per warp pass x threads per block x payload stages). */
int gw_autotune(gw_engine* e, int32_t K);

/* Selects a batched shape by hand (the values gw_get_shape reports);
 * GW_ERR_ARG when no such compiled shape exists or it does not fit. */
int gw_set_shape(gw_engine* e, int32_t kind, int32_t points_per_pass, int32_t threads, int32_t stages);

/* The K = 1 kernel: 0 = one block pipeline per tile (k_plain), 1 =
 * warp-specialised (k_plain_ws: six warps evaluate the next tile's dials while
 * two form the current tile's products and bin partials), 2 = the same with
 * eight evaluator warps.  gw_autotune(e, 1) times them and keeps the fastest.
 * Performance only: results are identical. */
int gw_set_plain_kernel(gw_engine* e, int32_t kind);
int gw_get_plain_kernel(const gw_engine* e, int32_t* kind);

/* Copies the batched shape in use out: kernel family (0 = lanes over points,
 * 1 = threads over dials, 3 = warp-specialised threads over dials for small
 * K), parameter points per pass, threads per block, payload stages. */
int gw_get_shape(const gw_engine* e, int32_t* kind, int32_t* points_per_pass, int32_t* threads, int32_t* stages);

/* The compiled batched shapes, for sweeps and tests.  gw_shape_count()
 * entries; gw_shape_at copies entry i out: family, points per pass, points
 * per thread (family 3: each evaluator thread takes all the points of a
 * pass), threads per block, payload stages and min_blocks (the CTAs per
 * SM its launch bounds ask the compiler to fit; 0 = the compiler's choice).
 * A shape may be compiled for several register targets; gw_set_shape takes
 * the first.  Such variants give identical results.  gw_set_shape_index
 * selects entry i (GW_ERR_ARG when out of range or it does not fit on an
 * SM); gw_get_shape_index reports the entry in use. */
int gw_shape_count(void);
int gw_shape_at(int32_t i, int32_t* kind, int32_t* points_per_pass, int32_t* points_per_thread, int32_t* threads,
                int32_t* stages, int32_t* min_blocks);
int gw_set_shape_index(gw_engine* e, int32_t i);
int gw_get_shape_index(const gw_engine* e, int32_t* i);

/* Cache::Manager::SetIsEventWeightCopyEnabled (CacheManager.h:119). */
int gw_set_event_weight_copy(gw_engine* e, int32_t enable);

/* Cache::Manager::CopyEventWeights (CacheManager.cpp:812-843): the per-event
 * weights of point 0 of the last gw_eval, in result order (n_results values).
 * Requires gw_set_event_weight_copy(e, 1) before the evaluation. */
int gw_get_event_weights(gw_engine* e, double* weights);

/* Cache::Manager::GetResidentMemory (CacheManager.h:192): device bytes held. */
int gw_resident_memory(const gw_engine* e, int64_t* bytes);

/* Measurement hooks (no reference counterpart; the reference keeps averaged
 * host timers, CacheManager.h:131-135).  With profiling on, every evaluation
 * records CUDA events on its launch stream around the weights kernel. */
int gw_set_profiling(gw_engine* e, int32_t on);
/* Sum of the weights-kernel durations (ms) and counts since the last read;
 * kernel_launches counts every engine kernel launched.  Resets the sums. */
int gw_read_profile(gw_engine* e, double* weights_ms, int64_t* weights_launches, int64_t* kernel_launches);

/* Per-bin likelihood terms, each bin as JointProbabilityBase::eval(const
 * SamplePair&, int) takes it (JointProbabilityBase.h:37-43 for
 * GW_LLH_POISSON, PoissonLogLikelihood.h:19-53; BarlowBeestonBanff2022.h:92-294
 * for GW_LLH_BARLOW_BEESTON_OA2021) from a histogram holding data[i], pred[i]
 * (sum of weights) and sqrt_sum_w2[i] (sqrt of the sum of squared weights),
 * evaluated on the device by the functions gw_eval's reduction sums.  Host
 * arrays of n values; out[i] = the bin's term, +inf (or NaN) where the
 * reference's default configuration throws (its throwIfInfLlh = false value). */
int gw_llh_bins(int32_t llh_type, const double* data, const double* pred, const double* sqrt_sum_w2, int32_t n,
                double* out);

/* Likelihood from bin sums the caller holds on the device, with no device
 * allocation.  No counterpart in the reference.  For callers that cannot call
 * cudaMalloc: code running inside a framework that owns the GPU's memory (a
 * caching allocator or a fitter's pool), or per-evaluation callbacks that must
 * not let cudaMalloc/cudaFree synchronise the device.
 *   d_sums, d_sums2 [K * n_bins]  sum of w and of w^2 per bin (device)
 *   d_data          [n_bins]      observed counts (device)
 *   d_llh           [K]           output: the summed per-bin likelihood (device)
 * Same per-bin terms and reduction order as gw_eval's llh_stat.  Scratch is a
 * fixed array inside the library (65536 block partials + 4096 counters, about
 * 528 KiB per GPU, held until exit): K <= 4096 and K * ceil(n_bins/256) <=
 * 65536, else GW_ERR_LIMIT.  All calls share that array: calls that overlap on
 * the GPU race.  The first call on a device looks up the array's address and
 * keeps it for the rest of the process; make it before any stream capture.
 * cudaDeviceReset destroys the context that address belongs to, so do not
 * call this on a device after a reset of that device in the same process.
 * Asynchronous on `stream`. */
int gw_llh_noalloc(const double* d_sums, const double* d_sums2, const double* d_data, int32_t n_bins, int32_t K,
                   int32_t llh_type, double* d_llh, void* stream);

/* Failure-path self-test (no reference counterpart): launches one block whose
 * bounded wait on a bulk-copy barrier cannot complete, with limit_us (<= 1 s)
 * as the limit.  timed_out = 1 when the wait gave up and reported it. */
int gw_selftest_wait_timeout(uint32_t limit_us, int32_t* timed_out);

/* FP32 FMA throughput of the device in TFLOP/s (independent FMA chains in
 * registers, best of four launches): the denominator of the compute roofline
 * of the batched kernels.  No reference counterpart. */
int gw_measure_fp32_peak(int32_t device, double* tflops);

/* Layout facts for measurement: tiles, dials, payload bytes, algorithmic
 * bytes read per evaluation pass. */
typedef struct gw_layout_info {
  int64_t n_tiles;
  int64_t n_dials;
  int64_t payload_bytes;
  int64_t header_bytes;
  int64_t event_bytes;
  int64_t partial_slots;
  int64_t dials_by_type[11];
} gw_layout_info;
int gw_get_layout(const gw_engine* e, gw_layout_info* info);

/* ---- learned surrogate: BF16 MLP on tensor cores (no reference counterpart) ----
 * A fully connected network dims[0] -> dims[1] -> ... -> dims[n_layers] with
 * SiLU between layers and a linear output, BF16 weights and activations with
 * FP32 accumulation (tcgen05), FP32 master weights updated by Adam.  It maps a
 * (standardised) parameter vector to predicted (standardised) log bin rates
 * and serves as the first stage of the delayed-acceptance sampler.  Widths and
 * batches must be multiples of 8. */
typedef struct gwm_net gwm_net;
int gwm_create(const int32_t* dims, int32_t n_layers, int32_t batch_max, int32_t device, gwm_net** net);
int gwm_destroy(gwm_net* net);
int gwm_last_error(const gwm_net* net, char* buf, size_t len);
/* Layer l weights w [dims[l+1] x dims[l]] row-major and bias b [dims[l+1]] (host FP32). */
int gwm_set_layer(gwm_net* net, int32_t layer, const float* w, const float* b);
int gwm_get_layer(gwm_net* net, int32_t layer, float* w, float* b);
/* y [B x dims[n]] = net(x [B x dims[0]]); FP32, host pointers or (device_ptrs != 0) device pointers. */
int gwm_forward(gwm_net* net, const float* x, int32_t B, float* y, int32_t device_ptrs);
/* One Adam step (beta 0.9 / 0.999) on the mean squared error of the batch; loss optional. */
int gwm_train_step(gwm_net* net, const float* x, const float* t, int32_t B, float lr, int32_t device_ptrs,
                   float* loss);
/* Gradients of the mean squared error of a batch, without updating (host arrays per layer). */
int gwm_gradients(gwm_net* net, const float* x, const float* t, int32_t B, float* const* grad_w,
                  float* const* grad_b, float* loss);
/* Surrogate head: inputs are standardised as (theta - in_mean) / in_scale
 * [dims[0]]; predicted log rate = base_b + base_w x + out_mu + out_sd * net(x)
 * (base_w [dims[n] x dims[0]], FP32); Sum w^2 is modelled as ratio * rate; data
 * [dims[n]] are the observed counts. */
int gwm_set_head(gwm_net* net, const float* in_mean, const float* in_scale, const float* base_w,
                 const float* base_b, const float* out_mu, const float* out_sd, const float* ratio,
                 const double* data);
/* Additive head: predicted log rate = base_b + sum_k interp_k(x_k) + out_mu +
 * out_sd * net(x), x = (theta - in_mean) / in_scale, with interp_k linear
 * between `nodes` (>= 2) equally spaced values base_tab[k][0..nodes-1][bin]
 * ([dims[0] x nodes x dims[n]], FP32) over x_k in [-lim, lim] and constant
 * outside; Sum w^2 = exp(ratio_b + ratio_w x) * rate (ratio_w [dims[n] x
 * dims[0]] optional, ratio_b [dims[n]] the log of the ratio). */
int gwm_set_head_additive(gwm_net* net, const float* in_mean, const float* in_scale, int32_t nodes, float lim,
                          const float* base_tab, const float* base_b, const float* out_mu, const float* out_sd,
                          const float* ratio_w, const float* ratio_b, const double* data);
/* Surrogate statistical likelihood (GW_LLH_*) of B points theta [B x dims[0]]
 * (host FP64) -> llh [B] (host); log_rates [B x dims[n]] optional. */
int gwm_predict(gwm_net* net, const double* theta, int32_t B, int32_t llh_type, double* llh, double* log_rates);
/* Training set held on the device: room for n_max points (clears the set). */
int gwm_train_reserve(gwm_net* net, int64_t n_max);
int gwm_train_size(gwm_net* net, int64_t* count);
/* Appends K <= batch_max points theta [K x dims[0]] (host FP64) and their bin
 * sums [K x dims[n]] (FP64; device memory when sums_on_device != 0).  The
 * target is the standardised residual of log(sums) after the head's affine
 * base, so gwm_set_head comes first. */
int gwm_train_append(gwm_net* net, const double* theta, const double* sums, int32_t K, int32_t sums_on_device);
/* As gwm_train_append, with the sums computed by the exact engine on the
 * device (gw_eval_device on the network's stream); K <= the engine's k_max. */
int gwm_train_append_eval(gwm_net* net, gw_engine* e, const double* theta, int32_t K);
/* Rows [first, first + count) of the set to the host: x [count x dims[0]]
 * standardised inputs, t [count x dims[n]] targets (either may be null). */
int gwm_train_read(gwm_net* net, int64_t first, int32_t count, float* x, float* t);
/* epochs x floor(size / batch) Adam steps over seeded per-epoch permutations
 * of the device-resident set, learning rate cosine-decayed lr0 -> lr_min;
 * losses [epochs] (optional) = mean loss per epoch. */
int gwm_train_epochs(gwm_net* net, int32_t epochs, int32_t batch, float lr0, float lr_min, uint64_t seed,
                     float* losses);
/* Stage 1 of the delayed-acceptance sampler on the device: random-walk
 * Metropolis sub-chains on f_s = surrogate statistical LLH + prior penalty
 * (GUNDAM's -2 log L convention; accept when log u < -(f' - f) / 2).
 * gwm_set_chain: proposal Cholesky factor L [P x P] (lower, row-major) and the
 * Gaussian prior (mean [P], inverse covariance [P x P]; both null: none),
 * P = dims[0] <= 1024.  gwm_substeps: n_sub steps for C <= batch_max chains from
 * theta0 [C x P] with values f0 [C] (null: evaluated first); writes the end
 * points phi [C x P], fphi [C] and the accepted sub-steps n_acc [C] (optional).
 * Normals and uniforms come from a counter-based hash of (seed, step, chain). */
int gwm_set_chain(gwm_net* net, const double* prop_chol, const double* prior_mean, const double* prior_icov);
int gwm_substeps(gwm_net* net, const double* theta0, const double* f0, int32_t C, int32_t n_sub, int32_t llh_type,
                 uint64_t seed, double* phi, double* fphi, int32_t* n_acc);
/* Value and gradient of the surrogate -2 log L (plus the prior penalty of
 * gwm_set_chain, when given) at C <= batch_max points theta [C x P] (host
 * FP64): f [C], grad [C x P] (host).  The gradient runs back through the
 * likelihood terms (closed-form derivatives), the base, the sum-of-w^2 model
 * and the network (tcgen05 backward GEMMs).  A deterministic function of the
 * point, so a leapfrog integrator built on it is exactly reversible. */
int gwm_value_grad(gwm_net* net, const double* theta, int32_t C, int32_t llh_type, double* f, double* grad);
/* The tensor-core GEMM alone: C [M x N] = A [M x K] * B [N x K]^T, BF16 in (raw bits), FP32 out, host arrays. */
int gwm_gemm_test(const uint16_t* A, const uint16_t* B, int32_t M, int32_t N, int32_t K, float* C);

#ifdef __cplusplus
}
#endif

#endif /* GW_H */
