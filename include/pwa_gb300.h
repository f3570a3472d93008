/*
 * pwa_gb300.h -- C ABI of the GB300-native extended-likelihood engine.
 *
 * The engine replaces the hot path of ROOTPWA's
 *   rpwa::pwaLikelihood<std::complex<double>>   (partialWaveFit/pwaLikelihood.h:66-320)
 *   rpwa::ampIntegralMatrix                      (decayAmplitude/ampIntegralMatrix.h:67-173)
 * with hand-written sm_103a CUDA kernels.  Every entry point mirrors one
 * reference method (cited beside it) with the same argument meaning, the same
 * call order and the same semantics; ROOT/Boost types are replaced by plain
 * pointers and sizes.
 *
 * Conventions
 *   - Every function returns an int status (PWA_SUCCESS == 0).  The reference
 *     reports setup failures as `false` + printErr and evaluation before
 *     finishInit() as a bare `throw;` (pwaLikelihood.cc:177-180); here both are
 *     status codes, and pwa_last_error() returns the message of the calling
 *     thread's last failure.
 *   - Sizes are 64-bit where they count events.
 *   - Complex numbers are interleaved (re, im) pairs: complex128 = 2 doubles,
 *     complex64 = 2 floats.
 *   - Parameter arrays follow the reference's function-parameter layout
 *     (pwaLikelihood.cc:1487-1556): for rank r, reflectivity (negative first),
 *     wave w in wave-list order: w < r absent, w == r one real parameter,
 *     w > r (Re, Im); the flat wave's real amplitude is the last parameter.
 *   - A handle may be used by one host thread at a time (the reference's
 *     evaluation methods write mutable caches and are not thread-safe either,
 *     pwaLikelihood.h:311-319).  Different handles are independent.
 */
#ifndef PWA_GB300_H
#define PWA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PWA_GB300_ABI_VERSION 1

typedef struct pwa_likelihood pwa_likelihood;
typedef struct pwa_integral   pwa_integral;

enum pwa_status {
	PWA_SUCCESS                = 0,
	PWA_ERROR_INVALID_ARGUMENT = 1,  /* null pointer, size mismatch, unknown wave */
	PWA_ERROR_INVALID_STATE    = 2,  /* call out of the reference's setup order */
	PWA_ERROR_CUDA             = 3,  /* a CUDA runtime call failed */
	PWA_ERROR_OUT_OF_MEMORY    = 4,
	PWA_ERROR_DEVICE_TIMEOUT   = 5,  /* a bounded device-side wait expired */
	PWA_ERROR_IO               = 6,  /* file could not be read or written */
	PWA_ERROR_UNSUPPORTED      = 7,  /* shape outside the compiled kernel variants */
	PWA_ERROR_NUMERICAL        = 8   /* e.g. singular Hessian in CovarianceMatrix */
};

/* pwaLikelihood::priorEnum (pwaLikelihood.h:108-111) */
enum pwa_prior { PWA_PRIOR_FLAT = 0, PWA_PRIOR_HALF_CAUCHY = 1 };

/* element type and residence of amplitude arrays handed to the engine */
enum pwa_amp_type { PWA_COMPLEX64 = 0, PWA_COMPLEX128 = 1 };
enum pwa_memory   { PWA_MEMORY_HOST = 0, PWA_MEMORY_DEVICE = 1 };

/* cross-event reduction of the FdF kernel (exact fixed point across blocks
 * in every mode).  Within a block each lane sums its events of a tile in
 * FP32; across tiles:
 *   PWA_REDUCE_FP64        FP32 partials of 32 tiles folded into FP64 (default)
 *   PWA_REDUCE_KAHAN_FP32  every tile's partial added to compensated FP32 sums
 *   PWA_REDUCE_FP32        plain FP32 sums over all of a lane's tiles
 * The two FP32 modes run the main kernel variant (not the fused-gradient one). */
enum pwa_reduction { PWA_REDUCE_FP64 = 0, PWA_REDUCE_KAHAN_FP32 = 1, PWA_REDUCE_FP32 = 2 };

/* arithmetic of the integral-matrix Gram kernel */
enum pwa_precision {
	PWA_PRECISION_FP64      = 0,  /* FP64 SIMT products and sums (slow on GB300; the accuracy reference) */
	PWA_PRECISION_FP32      = 1,  /* FP32 SIMT FMA, FP64 across chunks */
	PWA_PRECISION_TF32      = 2,  /* tcgen05 kind::tf32, FP32 accumulate in TMEM, FP64 across CTAs */
	PWA_PRECISION_TF32X3    = 3,  /* tcgen05 tf32 split hi+lo (3 products), FP32 accumulate, FP64 across CTAs */
	PWA_PRECISION_BF16X3    = 4   /* tcgen05 kind::f16 bf16 split hi+lo (3 products), FP32 accumulate */
};

/* function-call statistics, pwaLikelihood::functionCallEnum (pwaLikelihood.h:89-96) */
enum pwa_call { PWA_CALL_FDF = 0, PWA_CALL_GRADIENT = 1, PWA_CALL_DOEVAL = 2, PWA_CALL_DODERIVATIVE = 3,
                PWA_CALL_HESSIAN = 4 };

/* ------------------------------------------------------------------------ */
/* library                                                                   */
/* ------------------------------------------------------------------------ */
int         pwa_abi_version(void);
const char* pwa_last_error(void);
/* number of CUDA kernels this library launched since load (all handles) */
uint64_t    pwa_kernel_launch_count(void);

/* ------------------------------------------------------------------------ */
/* ampIntegralMatrix                                                          */
/* ------------------------------------------------------------------------ */
/* ampIntegralMatrix() (ampIntegralMatrix.cc:66-79) */
int pwa_integral_create(pwa_integral** out);
int pwa_integral_destroy(pwa_integral* I);
/* operator= (ampIntegralMatrix.cc:107-123) */
int pwa_integral_copy(pwa_integral* dst, const pwa_integral* src);
/* setWaveNames (ampIntegralMatrix.cc:255-277) */
int pwa_integral_set_wave_names(pwa_integral* I, uint32_t nWaves, const char* const* waveNames);
/*
 * integrate (ampIntegralMatrix.cc:300-489), on the GPU.
 * amps: [wave][event][subAmp] complex, host or device memory.  The reference
 * reads one ROOT tree per wave; here the waves are the rows of one array.
 * weights: optional importance-sampling weights w in the order the reference
 * reads its weight file: one per event that passes the bin selection, each
 * event entering with 1/w and the matrix renormalised by the mean of 1/w
 * (:419-429, :477-483).  inBin: optional per-event on-the-fly bin flag
 * (the reference's eventMeta + otfBin test, :411-416).  maxNmbEvents <= 0
 * uses all events.
 */
int pwa_integral_integrate(pwa_integral* I, uint32_t nWaves, const char* const* waveNames, const void* amps,
                           uint64_t nEvents, uint32_t nSubAmps, int ampType, int memory, const double* weights,
                           uint64_t nWeights, const uint8_t* inBin, int64_t maxNmbEvents, int precision);
/* addEvent (ampIntegralMatrix.cc:280-297): amps = nWaves complex128 in wave order */
int pwa_integral_add_event(pwa_integral* I, const double* amps);
/* element (ampIntegralMatrix.cc:238-252): raw sum / nmbEvents */
int pwa_integral_element(const pwa_integral* I, uint32_t i, uint32_t j, double* re, double* im);
/* matrix() (ampIntegralMatrix.h:114-117): raw sums, nWaves x nWaves complex128 row-major */
int pwa_integral_matrix(const pwa_integral* I, double* out);
int pwa_integral_set_matrix(pwa_integral* I, const double* in);
/* nmbWaves / nmbEvents / setNmbEvents (ampIntegralMatrix.h:99-103) */
int pwa_integral_nmb_waves(const pwa_integral* I, uint32_t* n);
int pwa_integral_nmb_events(const pwa_integral* I, uint64_t* n);
int pwa_integral_set_nmb_events(pwa_integral* I, uint64_t n);
/* waveIndex / waveName (ampIntegralMatrix.cc:195-216) */
int pwa_integral_wave_name(const pwa_integral* I, uint32_t i, char* buf, uint32_t bufLen);
int pwa_integral_wave_index(const pwa_integral* I, const char* name, uint32_t* index);
/* containsWave (ampIntegralMatrix.cc:188-191) */
int pwa_integral_contains_wave(const pwa_integral* I, const char* name, int* contains);
/* hasIdenticalWaveSet (ampIntegralMatrix.cc:633-646) and operator ==
 * (ampIntegralMatrix.h:179-195: same waves, same event count, equal raw sums
 * matched by wave name); either output may be NULL */
int pwa_integral_compare(const pwa_integral* I, const pwa_integral* other, int* identicalWaveSet, int* equal);
/* clear (ampIntegralMatrix.cc:93-103) */
int pwa_integral_clear(pwa_integral* I);
/* operator+= / -= / *= / /= (ampIntegralMatrix.cc:126-185) */
int pwa_integral_add(pwa_integral* I, const pwa_integral* other);
int pwa_integral_subtract(pwa_integral* I, const pwa_integral* other);
int pwa_integral_scale(pwa_integral* I, double factor);
int pwa_integral_divide(pwa_integral* I, double factor);
/* renormalize (ampIntegralMatrix.cc:492-500) */
int pwa_integral_renormalize(pwa_integral* I, uint64_t nmbEventsRenorm);
/* writeAscii / readAscii (ampIntegralMatrix.cc:503-570, file variants :573-608) */
int pwa_integral_read_ascii(pwa_integral* I, const char* path);
int pwa_integral_write_ascii(const pwa_integral* I, const char* path);
/*
 * No reference counterpart: the raw sums of integrate()'s Gram product
 * (ampIntegralMatrix.cc:408-469), I_ij = sum_k w_k A_ik conj(A_jk), from
 * device memory to device memory, allocating nothing.  amps: complex64
 * [nWaves][ldK] on the current device (nK events used per row); weights:
 * NULL or nK doubles on the device; out: nWaves x nWaves complex128
 * row-major on the device, full Hermitian matrix of raw sums (divide by the
 * event count for element()).  precision: PWA_PRECISION_FP64 or
 * PWA_PRECISION_FP32 (SIMT kernels).  Asynchronous on `stream`.
 * Partial sums go to a fixed 32 MiB device array (no cudaMalloc, no cudaFree,
 * no host synchronisation), for callers that must not allocate, e.g. one
 * integral per kinematic bin issued back to back on several streams, where a
 * cudaFree would synchronise the whole device.  Limits: nWaves <= 256
 * (PWA_GRAM_NOALLOC_MAX_WAVES); larger sets return PWA_ERROR_INVALID_ARGUMENT.  The first
 * call on a device (that device current) resolves the array's address and
 * has to precede any stream capture; the address it caches stays valid for
 * the life of the device's primary context (not across cudaDeviceReset).
 * Calls that overlap in time share the array and race: order them on one
 * stream.
 */
#define PWA_GRAM_NOALLOC_MAX_WAVES 256
int pwa_gram_device_noalloc(const void* amps, uint64_t nK, uint64_t ldK, uint32_t nWaves, const double* weights,
                            int precision, double* out, void* stream);
/*
 * No reference counterpart: the Gram sums of many bins in one call, for the
 * moment features of the learned warm start (the data-averaged
 * M_ij = <A_i conj(A_j)> of every kinematic bin); nWaves <= 1024.  amps[b]: complex64
 * [nWaves][nEvents[b]] contiguous on the current device; outGram:
 * nBins x nWaves x nWaves complex128 raw sums sum_k A_ik conj(A_jk) on the
 * device; outSums: NULL or nBins x nWaves complex128 raw sums sum_k A_ik
 * (compensated FP32 per thread, FP64 across threads).
 * precision: PWA_PRECISION_FP32 (SIMT) or a tensor-core precision
 * (PWA_PRECISION_TF32, _TF32X3, _BF16X3; bins whose rows are not 16-byte
 * aligned, i.e. an odd nEvents[b] or base, are first copied into an aligned
 * buffer; bins under 128 events use the FP32 SIMT kernel).  The kernels
 * are ordered on `stream`; the call allocates its
 * partial-sum and alignment buffers and returns after the stream has
 * completed them.
 */
int pwa_gram_device_batch(const void* const* amps, const uint64_t* nEvents, uint32_t nBins, uint32_t nWaves,
                          int precision, double* outGram, double* outSums, void* stream);

/* ------------------------------------------------------------------------ */
/* pwaLikelihood                                                              */
/* ------------------------------------------------------------------------ */
/* pwaLikelihood() (pwaLikelihood.cc:133-160); binds to the current CUDA device */
int pwa_likelihood_create(pwa_likelihood** out);
/* ~pwaLikelihood (pwaLikelihood.cc:163-167) */
int pwa_likelihood_destroy(pwa_likelihood* L);
/* useNormalizedAmps (pwaLikelihood.h:210) */
int pwa_likelihood_use_normalized_amps(pwa_likelihood* L, int flag);
/* setPriorType / setCauchyWidth (pwaLikelihood.h:212-215) */
int pwa_likelihood_set_prior_type(pwa_likelihood* L, int priorType);
int pwa_likelihood_set_cauchy_width(pwa_likelihood* L, double width);
/* normalizedAmpsUsed, priorType, cauchyWidth (pwaLikelihood.h:216-224); any
 * output may be NULL */
int pwa_likelihood_options(const pwa_likelihood* L, int* useNormalizedAmps, int* priorType, double* cauchyWidth);
/* dLcache (pwaLikelihood.h:200): grad [P] of the last FdF / Gradient call
 * (PWA_ERROR_INVALID_STATE before one) */
int pwa_likelihood_deriv_cache(const pwa_likelihood* L, double* grad);
/* clear (pwaLikelihood.cc:1670-1674): releases the device amplitude store;
 * evaluation is refused until the amplitudes are added and finishInit is
 * called again */
int pwa_likelihood_clear(pwa_likelihood* L);
/* No reference counterpart: event-sharded evaluation across processes (one
 * likelihood per process over a contiguous share of the data events).  Only
 * the root shard adds the normalisation term (with nEvt = totalEvents when
 * the amplitudes are not normalised) and the prior; the sum of all shards'
 * f and gradients (one all-reduce of P + 1 doubles) is the full FdF. */
int pwa_likelihood_set_shard(pwa_likelihood* L, uint64_t totalEvents, int root);
/* engine options without reference counterpart: CUDA stream of all launches,
 * cross-event reduction mode */
int pwa_likelihood_set_stream(pwa_likelihood* L, void* cudaStream);
int pwa_likelihood_set_reduction(pwa_likelihood* L, int reduction);
/* autotuner (no reference counterpart; the reference's CUDA path sized its
 * grid by an occupancy heuristic, cuda/likelihoodInterface.cu:304-360):
 * when enabled (default), finishInit times every compiled pipeline depth of
 * the FdF kernel on the handle's data and keeps the fastest; the choice is
 * cached per shape for the process.  pwa_likelihood_plan reports the plan in
 * use (events per tile = the amplitude store's block size, 128 or 64). */
int pwa_likelihood_set_autotune(pwa_likelihood* L, int enable);
int pwa_likelihood_plan(const pwa_likelihood* L, int* tileEvents, int* stages, int* blocks);
/* selects the pipeline depth by hand after finishInit (2..4 as shared memory allows) */
int pwa_likelihood_set_plan(pwa_likelihood* L, int stages);
/* events per block of the amplitude store (and FdF tile): 64 or 128, 0 for
 * the automatic choice (128 when two tiles fit in shared memory); before the
 * first addAmplitude().  Batched fits need 128. */
int pwa_likelihood_set_store_block(pwa_likelihood* L, uint32_t events);
/* FdF kernel variant: 1, 2 or 4 events per lane in the coherent-sum phase
 * (adjacent events share each V load; 2 and 4 read them with 128-bit loads;
 * 4 needs rank <= 2 and 128-event tiles), 3 the fused-gradient kernel (each
 * warp contracts its own events' gradient from registers; rank <= 2,
 * 128-event tiles), 5 the narrow kernel for small wave sets (one event per
 * thread, rank x waves <= 16: rank 1 up to 16 waves, rank 2 up to 8); 0
 * keeps the current one.  The autotuner times all that fit. */
int pwa_likelihood_set_plan_variant(pwa_likelihood* L, int stages, int phase1Events);
int pwa_likelihood_plan_variant(const pwa_likelihood* L, int* phase1Events);
/*
 * init (pwaLikelihood.cc:1050-1063 with readWaveList :1443-1484 and
 * buildParDataStruct :1487-1556).  The reference takes wave descriptions and
 * derives each wave's reflectivity from its decay topology; here the
 * reflectivity (+1 / -1) is passed directly, in wave-list order.
 */
int pwa_likelihood_init(pwa_likelihood* L, uint32_t nWaves, const char* const* waveNames,
                        const int32_t* reflectivities, const double* thresholds, uint32_t rank,
                        double massBinCenter);
/* addNormIntegral (pwaLikelihood.cc:1066-1083) */
int pwa_likelihood_add_norm_integral(pwa_likelihood* L, const pwa_integral* normMatrix);
/* addAccIntegral (pwaLikelihood.cc:1086-1107); like the reference it sets the
 * argument's nmbEvents to the number of generated events */
int pwa_likelihood_add_acc_integral(pwa_likelihood* L, pwa_integral* accMatrix, uint64_t accEventsOverride);
/* addAmplitude (pwaLikelihood.cc:1110-1288): one wave's decay amplitudes for
 * all data events, from host or device memory; normalised on upload */
int pwa_likelihood_add_amplitude(pwa_likelihood* L, const char* waveName, const void* amps, uint64_t nEvents,
                                 int ampType, int memory);
/* setOnTheFlyBinning (pwaLikelihood.cc:1391-1440): keep only the events of
 * the data file whose binning variables all satisfy lower[v] <= x_v <
 * upper[v], in file order.  binVars[v] points to nFileEvents doubles (host or
 * device memory); the selection runs on the GPU.  Call after
 * addAccIntegral() and before addAmplitude(); addAmplitude() then takes the
 * whole file's nFileEvents amplitudes and keeps the selected ones. */
int pwa_likelihood_set_otf_binning(pwa_likelihood* L, uint32_t nVars, const double* lower, const double* upper,
                                   const double* const* binVars, uint64_t nFileEvents, int memory);
/* number of data events selected by the on-the-fly binning (0 when unset) */
int pwa_likelihood_otf_selected(const pwa_likelihood* L, uint64_t* nSelected);
/* Raw amplitude files.  No reference counterpart as a format: they replace
 * the per-wave ROOT trees of amplitudeTreeLeaf objects
 * (storageFormats/amplitudeTreeLeaf.h:51-118) read by addAmplitude
 * (pwaLikelihood.cc:1110-1288) and the event-metadata binning variables read
 * by setOnTheFlyBinning (pwaLikelihood.cc:1391-1440).  One file holds N
 * events of one event file: W complex64 amplitude rows (one per wave, the
 * wave's N values contiguous) and V float64 binning-variable rows, after a
 * header with the names; the data block starts at a 4096-byte boundary.
 * amps is [nWaves][nEvents] complex64 and vars [nVars][nEvents] float64,
 * both host memory. */
int pwa_ampfile_write(const char* path, uint32_t nWaves, const char* const* waveNames, uint64_t nEvents,
                      const void* amps, uint32_t nVars, const char* const* varNames, const double* vars);
int pwa_ampfile_info(const char* path, uint32_t* nWaves, uint64_t* nEvents, uint32_t* nVars);
/* name of wave i (isVariable = 0) or of binning variable i (isVariable = 1) */
int pwa_ampfile_name(const char* path, int isVariable, uint32_t i, char* buf, uint32_t bufLen);
/* addAmplitude for every wave of the wave list from amplitude files, the
 * files' events concatenated in the order given, with on-the-fly binning on
 * the named variables when nBinVars > 0 (lower <= x < upper for each).  The
 * files are streamed through pinned buffers into device memory; the
 * selection and gather run on the GPU.  Call after addAccIntegral() and
 * before finishInit(), instead of addAmplitude(). */
int pwa_likelihood_load_amp_files(pwa_likelihood* L, uint32_t nFiles, const char* const* paths, uint32_t nBinVars,
                                  const char* const* binVarNames, const double* lower, const double* upper);
/* Autotuner cache (no reference counterpart; the reference picks its grid
 * by an occupancy heuristic, cuda/likelihoodInterface.cu:304-360).  The FdF
 * plans the autotuner measured in this process (per wave count, negative
 * waves, rank and event-count class) are written to / merged from a JSON
 * file tagged with the device name; a likelihood whose shape is in the cache
 * takes the cached plan at finishInit without timing runs.  Loading a cache
 * measured on another device model is refused. */
int pwa_autotune_cache_save(const char* path);
int pwa_autotune_cache_load(const char* path);
int pwa_autotune_cache_clear(void);
int pwa_autotune_cache_size(uint32_t* n);
/* Test hook (no reference counterpart): after n further device allocations
 * of the library, every allocation fails with PWA_ERROR_OUT_OF_MEMORY
 * without calling the CUDA allocator; n < 0 switches it off.  Exercises the
 * error paths of setup without exhausting a GPU. */
int pwa_debug_fail_alloc_after(int64_t n);
/* Test hook (no reference counterpart): runs one warp that waits, with the
 * kernels' own bounded-wait helper and a limit of limitMicroseconds
 * (1 .. 1,000,000), on an mbarrier armed for a transfer that is never
 * issued.  The wait expires without any fault and the call returns
 * PWA_ERROR_DEVICE_TIMEOUT, the status every streaming kernel reports when a
 * wait runs out; the context stays usable. */
int pwa_debug_stalled_wait(uint32_t limitMicroseconds);
/* finishInit (pwaLikelihood.cc:1291-1388) */
int pwa_likelihood_finish_init(pwa_likelihood* L);

/* accessors (pwaLikelihood.h:188-196, :163) */
int pwa_likelihood_nmb_pars(const pwa_likelihood* L, uint32_t* n);       /* NDim() */
int pwa_likelihood_nmb_pars_fixed(const pwa_likelihood* L, uint32_t* n);
int pwa_likelihood_nmb_events(const pwa_likelihood* L, uint64_t* n);
int pwa_likelihood_rank(const pwa_likelihood* L, uint32_t* r);
/* nmbWaves(reflectivity): 0 = all, > 0 positive, < 0 negative (pwaLikelihood.cc:1015-1024) */
int pwa_likelihood_nmb_waves(const pwa_likelihood* L, int reflectivity, uint32_t* n);
/* parameter(i) (pwaLikelihood.h:114-150): name as fitParameter::parName() */
int pwa_likelihood_parameter(const pwa_likelihood* L, uint32_t i, char* nameBuf, uint32_t bufLen, int* fixed,
                             int* realPart, int32_t* rank, double* threshold);
/* totAcc of the acceptance integral (pwaLikelihood.cc:1100) */
int pwa_likelihood_tot_acc(const pwa_likelihood* L, double* totAcc);

/* FdF (pwaLikelihood.cc:170-315): f and the full-length gradient */
int pwa_likelihood_fdf(pwa_likelihood* L, const double* par, double* f, double* grad);
/* DoEval (pwaLikelihood.cc:318-435) */
int pwa_likelihood_doeval(pwa_likelihood* L, const double* par, double* f);
/* Gradient (pwaLikelihood.cc:474-636) */
int pwa_likelihood_gradient(pwa_likelihood* L, const double* par, double* grad);
/* DoDerivative (pwaLikelihood.cc:438-471): cached gradient if par equals the
 * last evaluated point, else a full FdF */
int pwa_likelihood_doderivative(pwa_likelihood* L, const double* par, uint32_t index, double* d);
/* nPoints parameter vectors [nPoints][P] -> f[nPoints], grad[nPoints][P];
 * one FdF per point, launched back to back on the handle's stream */
int pwa_likelihood_fdf_batch(pwa_likelihood* L, uint32_t nPoints, const double* par, double* f, double* grad);
/* Device-resident FdF for device-side minimisers and graph capture: reads
 * P doubles at dPar, writes dOut[0] = f, dOut[1..P] = gradient, asynchronously
 * on `stream` (NULL = the handle's stream).  withGradient = 0 gives DoEval. */
int pwa_likelihood_fdf_device(pwa_likelihood* L, const double* dPar, double* dOut, int withGradient, void* stream);
/* Hessian (pwaLikelihood.cc:639-859): P x P row-major */
int pwa_likelihood_hessian(pwa_likelihood* L, const double* par, double* hessian);
/* CovarianceMatrix(hessian) (pwaLikelihood.cc:929-981) */
int pwa_likelihood_covariance_matrix(const pwa_likelihood* L, const double* hessian, double* covariance);
/* HessianEigenVectors (pwaLikelihood.cc:864-912, called by pwaFit.cc:308,
 * pwaNloptFit.cc:251 and pyInterface/module/_fit.py:197): eigenvalues and
 * eigenvectors of the Hessian [P][P] restricted to the free parameters.
 * eigenvalues [P]: the first *nFree entries, descending; eigenvectors [P][P]:
 * row k is the eigenvector of eigenvalue k in the full parameter space (zero
 * at fixed parameters; sign arbitrary).  Needs init() only. */
int pwa_likelihood_hessian_eigenvectors(const pwa_likelihood* L, const double* hessian, double* eigenvalues,
                                        double* eigenvectors, uint32_t* nFree);
/* CorrectParamSigns (pwaLikelihood.cc:984-1010) */
int pwa_likelihood_correct_param_signs(const pwa_likelihood* L, const double* par, double* out);
/* getIntegralMatrices (pwaLikelihood.cc:1579-1622): norm and acc as
 * n x n complex128 (n = nmbWaves + withFlat), phaseSpace as n doubles */
int pwa_likelihood_integral_matrices(const pwa_likelihood* L, double* norm, double* acc, double* phaseSpace,
                                     int withFlat);
/* buildProdAmpArrays (pwaLikelihood.cc:1626-1665): production amplitudes
 * (complex128, count = parameters without the flat imaginary slots) and
 * their parameter index pairs (im = -1 for real amplitudes); returns the count
 * in *nAmps.  Buffers must hold P entries. */
int pwa_likelihood_build_prod_amp_arrays(const pwa_likelihood* L, const double* par, double* prodAmps,
                                         int32_t* parIndices, uint32_t* nAmps, int withFlat);
/* functionCallInfo (pwaLikelihood.h:88-106): calls, total / event-loop /
 * normalisation seconds per call type */
int pwa_likelihood_func_call_info(const pwa_likelihood* L, int call, uint64_t* nCalls, double* totalTime,
                                  double* funcTime, double* normTime);
int pwa_likelihood_reset_func_call_info(pwa_likelihood* L);
/* Engine instrumentation without reference counterpart: when enabled, every
 * evaluation records CUDA events on its launch stream before and after the
 * fused FdF kernel (one launch per evaluation, the normalisation term and the
 * cross-block sums included).  pwa_likelihood_kernel_times waits for the
 * recorded events, returns the summed kernel duration in milliseconds
 * (finalizeMs is always 0: there is no second kernel) and the number of timed
 * evaluations, and clears the record.  At most 65536 evaluations are recorded
 * between two reads. */
int pwa_likelihood_set_timing(pwa_likelihood* L, int enable);
int pwa_likelihood_kernel_times(pwa_likelihood* L, double* eventKernelMs, double* finalizeMs, uint64_t* nTimed);

/* ------------------------------------------------------------------------ */
/* Batched multibin x multistart fits (no reference counterpart: the          */
/* reference fits one bin per process, pwaFit.py:18,51-57, and its start      */
/* points one after another, _fit.py:131-165)                                 */
/* ------------------------------------------------------------------------ */
typedef struct pwa_multibin pwa_multibin;
/* L-BFGS status of a problem (one bin x one start point) */
enum pwa_lbfgs_status { PWA_LBFGS_ACTIVE = 0, PWA_LBFGS_SEARCHING = 1, PWA_LBFGS_CONVERGED = 2,
                        PWA_LBFGS_MAX_ITER = 3, PWA_LBFGS_STALLED = 4, PWA_LBFGS_FAILED = 5,
                        PWA_LBFGS_FLOOR = 6 /* gradient norm stopped improving (rounding floor) */ };
int pwa_multibin_create(pwa_multibin** out);
int pwa_multibin_destroy(pwa_multibin* M);
/* adds a bin: a likelihood after finishInit (rank 1, one reflectivity, at
 * most 64 waves; every bin the same wave set and layout) with nStarts start
 * points; the likelihood must outlive the batch.  Problems are numbered bin
 * by bin, start by start. */
int pwa_multibin_add_bin(pwa_multibin* M, pwa_likelihood* L, uint32_t nStarts);
/* startGroup: starts evaluated together per amplitude tile (8 or 32);
 * L-BFGS memory; convergence when |grad| <= gtolAbs + gtolRel * max(1, |f|);
 * iteration limit per problem */
int pwa_multibin_set_options(pwa_multibin* M, uint32_t startGroup, uint32_t lbfgsMemory, double gtolAbs,
                             double gtolRel, uint32_t maxIter);
/* trace of the last fit: at each check (every sweepsPerGraph sweeps) the
 * seconds since the fit started and the accepted f of every problem
 * (f [check][Q]); returns the number of checks (copies at most maxChecks) */
int pwa_multibin_trace(const pwa_multibin* M, uint32_t maxChecks, double* seconds, double* f, uint32_t* nChecks);
/* a problem stops with PWA_LBFGS_FLOOR when its gradient norm has not
 * improved by 1% for this many iterations (default 50, 0 = never) */
int pwa_multibin_set_floor_window(pwa_multibin* M, uint32_t iterations);
/* tiles of 128 events per work item for bins of < 64, < 512 and >= 512 tiles */
int pwa_multibin_set_chunks(pwa_multibin* M, const uint32_t* tilesPerItem);
int pwa_multibin_chunks(const pwa_multibin* M, uint32_t* tilesPerItem);
/* autotuner: per bin size class in turn, the tiles per item with the fastest
 * evaluation sweep at x [Q][P] */
int pwa_multibin_autotune(pwa_multibin* M, const double* x);
int pwa_multibin_nmb_problems(const pwa_multibin* M, uint32_t* nProblems);
int pwa_multibin_nmb_pars(const pwa_multibin* M, uint32_t* nPars);
/* FdF of every problem: x [Q][P] -> f [Q], grad [Q][P] (host buffers) */
int pwa_multibin_fdf(pwa_multibin* M, const double* x, double* f, double* grad);
/* device time of one evaluation sweep of all problems at x (mean of reps) */
int pwa_multibin_sweep_ms(pwa_multibin* M, const double* x, uint32_t reps, double* ms);
/* L-BFGS of every problem from x0 [Q][P]: sweeps (one batched FdF + one
 * L-BFGS step for all active problems) run until no problem is active or
 * maxSweeps; with useGraph the sweeps are replayed from a CUDA graph of
 * sweepsPerGraph sweeps.  Outputs (host, any may be NULL): x [Q][P], f, gnorm,
 * status (pwa_lbfgs_status), iterations [Q], sweeps run. */
int pwa_multibin_fit(pwa_multibin* M, const double* x0, int useGraph, uint32_t sweepsPerGraph, uint32_t maxSweeps,
                     double* x, double* f, double* gnorm, int32_t* status, uint32_t* iterations, uint32_t* sweeps);
/* Checkpoint / resume of a batched fit (no reference counterpart; the
 * reference appends each finished fit to a ROOT tree, pwaFit.py:101-130).
 * The fit state (iterates, trial points, gradients, L-BFGS histories and
 * per-problem counters) lives on the device; save_state writes it to a file
 * (through path.tmp and a rename), load_state reads it back into a batch
 * with the same bins, starts and options, and resume continues the sweeps
 * from it, giving the same results bit for bit as a fit that was never
 * interrupted.  set_checkpoint makes fit/resume write the file every
 * `everySweeps` sweeps, between graph launches (0 switches it off). */
int pwa_multibin_save_state(pwa_multibin* M, const char* path);
int pwa_multibin_load_state(pwa_multibin* M, const char* path);
int pwa_multibin_resume(pwa_multibin* M, int useGraph, uint32_t sweepsPerGraph, uint32_t maxSweeps, double* x,
                        double* f, double* gnorm, int32_t* status, uint32_t* iterations, uint32_t* sweeps);
int pwa_multibin_set_checkpoint(pwa_multibin* M, const char* path, uint32_t everySweeps);
/* sweeps run since the fit started (including those before a saved state) */
int pwa_multibin_sweeps_done(const pwa_multibin* M, uint32_t* sweeps);

/* ------------------------------------------------------------------------ */
/* Learned warm start (no reference counterpart): a 3-layer perceptron        */
/* nIn -> nHidden1 -> nHidden2 -> nOut with relu, BF16 weights and            */
/* activations, FP32 accumulation and FP32 master weights, trained with Adam  */
/* on the mean squared error.  Parameters are laid out W1 [nHidden1][nIn], b1,*/
/* W2 [nHidden2][nHidden1], b2, W3 [nOut][nHidden2], b3 (FP32).               */
/* ------------------------------------------------------------------------ */
typedef struct pwa_mlp pwa_mlp;
/* He-normal weights from `seed`, zero biases */
int pwa_mlp_create(pwa_mlp** out, uint32_t nIn, uint32_t nHidden1, uint32_t nHidden2, uint32_t nOut, uint64_t seed);
int pwa_mlp_destroy(pwa_mlp* net);
int pwa_mlp_nmb_params(const pwa_mlp* net, uint64_t* n);
int pwa_mlp_get_params(const pwa_mlp* net, float* params);
/* sets the FP32 master weights (and their BF16 copy); resets Adam's moments */
int pwa_mlp_set_params(pwa_mlp* net, const float* params);
/* Y [B][nOut] = net(X [B][nIn]) (host buffers; X is rounded to BF16) */
int pwa_mlp_forward(pwa_mlp* net, const float* X, uint32_t B, float* Y);
/* mean squared error of net(X) against T [B][nOut] and its gradient in the
 * parameter layout (host buffers; loss and grad may be NULL) */
int pwa_mlp_gradient(pwa_mlp* net, const float* X, const float* T, uint32_t B, double* loss, float* grad);
/* Adam (lr, betas 0.9 / 0.999) over `epochs` shuffled passes of mini-batches
 * of `batch` samples; lossHistory [epochs] (may be NULL) gets the mean batch
 * loss of each epoch */
int pwa_mlp_train(pwa_mlp* net, const float* X, const float* T, uint64_t nSamples, uint32_t batch, uint32_t epochs,
                  float lr, uint64_t seed, double* lossHistory);

/* ------------------------------------------------------------------------ */
/* Decay amplitudes of three spinless final-state particles in the isobar    */
/* model, helicity or canonical formalism (the step before the likelihood:   */
/* replaces isobarAmplitude::amplitude, decayAmplitude/isobarAmplitude.h:80, */
/* isobarAmplitude.cc:98-262, isobarHelicityAmplitude.cc:64-195,             */
/* isobarCanonicalAmplitude.cc:64-190, for X -> isobar + bachelor,           */
/* isobar -> a + b).  Spins, projections and orbital                         */
/* angular momenta are integers in units of 1/2 (2J, 2M, 2L), as in the      */
/* reference.  FP64 on the GPU, one thread per event.                        */
/* ------------------------------------------------------------------------ */
typedef struct pwa_isobar pwa_isobar;
/* massDependence (decayAmplitude/massDependence.cc:169-862): flatMassDependence, binnedMassDependence,
 * relativisticBreitWigner, constWidthBreitWigner, rhoBreitWigner,
 * f0980BreitWigner, f0980FlatteBesII (fixed BES II parameters),
 * piPiSWaveAuMorganPenningtonM / Ves / Kachaev (fixed AMP parameters; for the
 * fixed-parameter forms mass and width are unused) */
enum pwa_mass_dependence {
	PWA_MASSDEP_FLAT = 0,
	PWA_MASSDEP_RELATIVISTIC_BW = 1,
	PWA_MASSDEP_CONST_WIDTH_BW = 2,
	PWA_MASSDEP_RHO_BW = 3,
	PWA_MASSDEP_F0980_BW = 4,
	PWA_MASSDEP_F0980_FLATTE = 5,
	PWA_MASSDEP_PIPI_S_AMP_M = 6,
	PWA_MASSDEP_PIPI_S_AMP_VES = 7,
	PWA_MASSDEP_PIPI_S_AMP_KACHAEV = 8,
	PWA_MASSDEP_BINNED = 9,           /* binnedMassDependence: 1 inside [binLower, binUpper), else 0 */
	PWA_MASSDEP_RHO_PRIME = 10,       /* rhoPrimeMassDep: fixed rho(1450) / rho(1700) mixture */
	PWA_MASSDEP_KPI_S_GLASS = 11,     /* KPiSGLASS: K pi S-wave, LASS form with massDepParams */
	PWA_MASSDEP_KPI_S_PALANO_PENNINGTON = 12 /* KPiSPalanoPennington: K pi / K eta K-matrix */
};
/* one wave: the content of a key file of a three-body decay
 * (decayAmplitude/waveDescription.cc:880-932) */
typedef struct pwa_isobar_wave {
	int32_t J, P, M, refl;            /* X: 2J, parity, 2M (>= 0 in the reflectivity basis), reflectivity */
	int32_t L, S;                     /* X -> daughter 1 + daughter 2: 2L, 2S */
	int32_t isobarJ, isobarL, isobarS; /* isobar 2J and its decay's 2L, 2S */
	int32_t massDependence;           /* enum pwa_mass_dependence of the isobar */
	double isobarMass, isobarWidth;   /* GeV/c^2 */
	int32_t isobarDaughter1, isobarDaughter2, bachelor; /* final-state slots 0..2; isobar daughter 1 is the analyser */
	int32_t bachelorFirst;            /* X-vertex daughter 1 (the analyser) is the bachelor rather than the isobar */
	int32_t isospin, isobarIsospin;   /* 2I of X and of the isobar (isospin symmetrisation only) */
	double binLower, binUpper;        /* PWA_MASSDEP_BINNED: the isobar mass bin [lower, upper) */
	double massDepParams[10];         /* PWA_MASSDEP_KPI_S_GLASS: a, r, M0, G0, phiF, phiR, phiRsin, F, R, MMax;
	                                     PWA_MASSDEP_KPI_S_PALANO_PENNINGTON: MMax (0: 2.4 GeV/c^2) */
} pwa_isobar_wave;
/* isobarHelicityAmplitude (decayAmplitude/isobarHelicityAmplitude.cc:64-195)
 * or isobarCanonicalAmplitude (decayAmplitude/isobarCanonicalAmplitude.cc:64-190) */
enum pwa_formalism { PWA_FORMALISM_HELICITY = 0, PWA_FORMALISM_CANONICAL = 1 };
int pwa_isobar_create(pwa_isobar** out);
int pwa_isobar_destroy(pwa_isobar* A);
/* three final-state particles: masses, species ids (equal ids are identical
 * particles, Bose-symmetrised) and the beam mass (GeV/c^2); energies follow
 * from the masses and momenta as in particle::setMomentum */
int pwa_isobar_set_final_state(pwa_isobar* A, uint32_t nFsParticles, const double* masses, const int32_t* species,
                               double beamMass);
/* isobarAmplitude::enableReflectivityBasis / enableBoseSymmetrization /
 * enableSpaceInversion / enableReflection (isobarAmplitude.h:68-75);
 * defaults 1, 1, 0, 0 */
int pwa_isobar_set_options(pwa_isobar* A, int reflectivityBasis, int boseSymmetrize, int spaceInversion,
                           int reflection);
/* helicity (the default) or canonical formalism */
int pwa_isobar_set_formalism(pwa_isobar* A, int formalism);
/* no reference counterpart: run on the caller's CUDA stream (NULL = the
 * default stream); calls with device buffers are then asynchronous in stream
 * order, calls with host buffers still return with the results in place */
int pwa_isobar_set_stream(pwa_isobar* A, void* cudaStream);
/* no reference counterpart: host-buffer calls process at most this many
 * events per device pass (0, the default: 1 GiB of device buffers) */
int pwa_isobar_set_chunk_events(pwa_isobar* A, uint64_t events);
/* isospin symmetrisation (isobarDecayTopology::getIsospinSymmetrization,
 * isobarDecayTopology.cc:505-630; isobarAmplitude::enableIsospinSymmetrization):
 * the final-state particles' 2I, 2I_3 and intrinsic parities; enabling it
 * needs them (it is off by default here, on in the reference, which takes the
 * isospins from its particle table) */
int pwa_isobar_set_isospins(pwa_isobar* A, const int32_t* isospin, const int32_t* isospinProj,
                            const int32_t* parity);
int pwa_isobar_enable_isospin_symmetrization(pwa_isobar* A, int flag);
int pwa_isobar_add_wave(pwa_isobar* A, const pwa_isobar_wave* wave);
int pwa_isobar_nmb_waves(const pwa_isobar* A, uint32_t* n);
/* number of symmetrisation terms (Bose times isospin) of one wave with the
 * current final state and options */
int pwa_isobar_nmb_sym_terms(const pwa_isobar* A, uint32_t wave, uint32_t* n);
/* amplitudes of every wave for nEvents events: beam momenta [3][nEvents]
 * (px, py, pz rows), final-state momenta [3 particles][3][nEvents], lab frame,
 * GeV/c; amps [wave][nEvents] of ampType: PWA_COMPLEX128 (FP64 arithmetic
 * throughout, like the reference) or PWA_COMPLEX64 (frames and kinematics in
 * FP64, the per-wave D functions, barrier factors and mass dependences in
 * FP32; the likelihood's amplitude store is complex64).  memory:
 * PWA_MEMORY_HOST or PWA_MEMORY_DEVICE for all three buffers. */
int pwa_isobar_amplitudes(pwa_isobar* A, const double* beam, const double* fs, uint64_t nEvents, void* amps,
                          int ampType, int memory);
/* calcAmplitudes (pyInterface/scripts/calcAmplitudes.py): the amplitudes of
 * every wave for host momenta (layout as above), computed on the GPU in slabs
 * and written as one raw amplitude file (pwa_ampfile_*): complex64 rows named
 * waveNames[W], binning variables "mass" (the final-state mass) and the
 * caller's nVars rows vars [nVars][nEvents] */
int pwa_isobar_write_amp_file(pwa_isobar* A, const char* path, const char* const* waveNames, const double* beam,
                              const double* fs, uint64_t nEvents, uint32_t nVars, const char* const* varNames,
                              const double* vars);
/* host utilities: clebschGordanCoeff (utilities/spinUtils.hpp:241-330),
 * dFunction (utilities/dFunction.hpp:52-170), barrierFactor with the
 * 0.1973 GeV/c scale (utilities/physUtils.hpp:200-275); arguments doubled */
int pwa_clebsch_gordan(int32_t j1, int32_t m1, int32_t j2, int32_t m2, int32_t J, int32_t M, double* out);
int pwa_wigner_d(int32_t j, int32_t m, int32_t n, double theta, double* out);
int pwa_barrier_factor(int32_t L, double q, double* out);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* PWA_GB300_H */
