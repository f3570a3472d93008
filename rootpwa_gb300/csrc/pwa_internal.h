// pwa_internal.h -- declarations shared by the host library and the CUDA
// kernels of the GB300 extended-likelihood engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

struct pwa_likelihood;

namespace pwa {

// status codes (same values as enum pwa_status in include/pwa_gb300.h)
enum {
	kOk = 0,
	kErrArg = 1,
	kErrState = 2,
	kErrCuda = 3,
	kErrOom = 4,
	kErrTimeout = 5,
	kErrIo = 6,
	kErrUnsupported = 7,
	kErrNumerical = 8
};

#define PWA_CHECK(expr)         \
	do {                        \
		const int _st = (expr); \
		if (_st != 0)           \
			return _st;         \
	} while (0)

// records the calling thread's last error; returns code
int setError(int code, const std::string& msg);
// checks a CUDA runtime result; records and returns kErrCuda on failure
int cudaCheck(cudaError_t e, const char* what);
// counts kernel launches (reported through pwa_kernel_launch_count)
void countLaunches(uint64_t n);

// Device-side error flags: a bounded wait expired; a shared-memory access
// failed its bounds check (builds with PWA_DEBUG_CHECKS only; the access is
// skipped).
enum { kDevErrTimeout = 1, kDevErrBounds = 2 };

// ---------------------------------------------------------------------------
// Amplitude store
// ---------------------------------------------------------------------------
// complex64 amplitudes in blocks of B events (B = 128, or 64 for wide wave
// sets).  Block b holds the W wave rows of its B events contiguously (waves of
// negative reflectivity first), so one bulk copy moves one tile.  Row w keeps
// event b*B + p at position (p + rot(w)) mod B with
// rot(w) = (B/32) * (w mod (512/B)).  In the FdF kernel's first phase a
// half-warp reads 512/B consecutive rows (w mod 512/B = 0, 1, ...) at the
// same B/32 events; the rotation puts those pieces at distinct offsets
// (B/32 events = 32 bytes apart for B = 128), so they fall on distinct
// shared-memory banks.  Rotations are even, so event pairs (p, p+1) with p
// even never wrap.  The last block is zero-padded.
__host__ __device__ inline uint32_t storeRot(uint32_t w, uint32_t B) { return (B / 32) * (w % (512 / B)); }

__host__ __device__ inline uint64_t storeIndex(uint32_t w, uint64_t e, uint32_t W, uint32_t B)
{
	const uint64_t b = e / B;
	const uint32_t p = (uint32_t)(e - b * B);
	return (b * W + w) * B + ((p + storeRot(w, B)) & (B - 1));
}

// ---------------------------------------------------------------------------
// Fused FdF / DoEval
// ---------------------------------------------------------------------------
struct FdfPlan {
	int E = 128;        // events per tile (= store block)
	int stages = 2;     // shared-memory pipeline depth
	int wpw = 2;        // wave bucket per warp (template)
	int phase1Events = 2;  // events per lane in the coherent-sum phase (1, 2 or 4; 3: fused-gradient variant; 5: narrow variant)
	int blocks = 0;     // grid size (persistent, <= #SMs)
	size_t smemBytes = 0;
};

struct FdfArgs {
	const float2* amps;      // tiled store (storeIndex)
	uint64_t nEvents;
	int W0, W, R, P;
	const double* par;       // device, [P]
	const int* slotRe;       // device, [R*W] parameter index of Re(V_rw) or -1
	const int* slotIm;       // device, [R*W] parameter index of Im(V_rw) or -1
	const double* accI;      // device, per reflectivity e: W_e x W_e complex128 (re, im) row-major, e=0 block first
	double nEvt, totAcc;     // normalisation factor (1 or N) and total acceptance
	int prior;               // 0 flat, 1 half-Cauchy
	double cauchyWidth;
	int withGrad;
	int reduction;           // 0 = FP64 across tiles, 1 = compensated FP32, 2 = plain FP32
	int nPartial;            // 2 + 2*R*W summed values (LL, sum c, gradient re/im per slot)
	unsigned long long* fixAcc;  // device, fdfAccumulatorWords(nPartial) 128-bit fixed-point totals, zero between launches
	double* nfAcc;           // device, [nPartial] totals of values outside the fixed-point range, zero between launches
	unsigned* counter;       // device, arrival counter, zero between launches
	unsigned* devErr;        // device error flags
	double* out;             // device, [P + 2]: f, gradient, device error status
	const int* active;       // device flag or null: when it is 0 the launch does nothing (batched fits)
};

// Store block size for a wave set: 128 when two 128-event tiles fit in shared
// memory, else 64.
int chooseStoreBlock(int W, int R, size_t maxSmem);
// All compiled pipeline depths for tiles of B events that fit, for the autotuner.
int planCandidates(int W0, int W, int R, int B, uint64_t nEvents, int numSMs, size_t maxSmem,
                   std::vector<FdfPlan>* out);
int launchFdf(const FdfPlan& plan, const FdfArgs& args, cudaStream_t s);
// 64-bit words of the FdF kernel's fixed-point accumulators (all replicas).
size_t fdfAccumulatorWords(int nPartial);
// Fused-gradient FdF variant (fdf_fused.cu, plan phase1Events == 3):
// 128-event tiles, rank 1 or 2, at most 16 negative and 104 positive waves.
// Dynamic shared memory it needs for `stages` stages, 0 when unsupported.
size_t fusedFdfSmem(int W0, int W, int R, int stages);
int launchFdfFused(const FdfPlan& plan, const FdfArgs& args, cudaStream_t s);
// Narrow FdF variant for small wave sets (fdf_narrow.cu, plan phase1Events
// == 5): one event per thread, 512-event tiles, rank x waves <= 16.
int narrowMaxWaves(int R);
size_t narrowFdfSmem(int W, int R, int stages);
uint64_t narrowFdfTiles(uint64_t nEvents);
int launchFdfNarrow(const FdfPlan& plan, const FdfArgs& args, cudaStream_t s);

// Converts one wave w of amplitudes (complex64 or complex128, device memory)
// into the tiled complex64 store, divided by `divisor` in FP64; sets *nonzero
// to 1 if any amplitude is non-zero.
int launchConvertRow(const void* src, int srcIsDouble, float2* store, uint32_t W, uint32_t w, uint32_t B, uint64_t n,
                     double divisor, unsigned* nonzero, cudaStream_t s);
// Converts amplitudes to complex64 rows [wave][event] of a plain array (integral input).
int launchConvertPlain(const void* src, float2* dst, uint64_t n, cudaStream_t s);

// ---------------------------------------------------------------------------
// Hessian event term
// ---------------------------------------------------------------------------
// For events [e0, e0 + slab) writes, per event t (column of the slab):
//   Y1 rows [0, nS):      d_s = S_{r(s),e(s)} conj(A_{w(s)})   (nS = R*W slots)
//   Y1 rows [nS, 2nS):    conj(d_s)
//   Y1 row 2nS:           1
//   Y2 rows [0, W):       A_w;   Y2 row W: 1
//   w1 = f^2, w2 = f with f = 2 / L (0 beyond nEvents)
// so that the weighted Gram matrices of Y1 and Y2 give every event sum of the
// analytic Hessian (partialWaveFit/pwaLikelihood.cc:676-735).
int launchHessPrep(const float2* amps, uint64_t nEvents, uint32_t B, uint64_t e0, uint64_t slab, int W0, int W,
                   int R, int P, const double* par, const int* slotRe, const int* slotIm, float2* Y1, float2* Y2,
                   double* w1, double* w2, cudaStream_t s);

// ---------------------------------------------------------------------------
// Integral matrix (Gram) kernels
// ---------------------------------------------------------------------------
struct GramArgs {
	const float2* amps;     // [W][K] complex64 (K = events x subamps), row stride ldK (elements)
	const double2* amps64;  // [W][K] complex128 alternative (FP64 precision)
	uint64_t K;
	uint64_t ldK;
	int W;
	const double* weightK;  // optional per-K weight (1/w, already expanded over subamps), or null
	double* partials;       // [chunks][W*W*2]
	int chunks;
	unsigned* devErr;
	// tensor-core Gram only: 0, or the element offset between two groups of
	// W / 2 rows each (the Gram of rows 0..W/2-1 and groupStride.. + W/2-1)
	uint64_t groupStride;
};
int launchGramSimt(const GramArgs& a, int precision, cudaStream_t s);
// out = (accumulate ? out : 0) + sum of chunk partials, mirrored to the lower triangle
int launchGramReduce(const double* partials, int chunks, int W, double* out, int accumulate, cudaStream_t s);
// out[w] = sum_k a[w][k] for W complex64 rows of n elements (row stride ld),
// FP64 (complex128 out[W])
int launchRowSums(const float2* a, uint64_t n, uint64_t ld, int W, double* out, cudaStream_t s);
// out (nOut x nOut complex) += blocks of the Gram blk of two row groups of G
// rows (groups a and b; see integral_kernels.cu)
int launchGramBlockAdd(const double* blk, int n2, int G, int a, int b, int nOut, int addAA, int addBB, double* out,
                       cudaStream_t s);
// tcgen05 tensor-core Gram; returns kErrUnsupported when the shape has no variant
int launchGramTc(const GramArgs& a, int precision, int numSMs, cudaStream_t s, double* out, double* scratch,
                 size_t scratchDoubles);
// FP32 words of per-CTA partial Grams launchGramTc needs
size_t gramTcScratchFloats(int W, int numSMs);

// ---------------------------------------------------------------------------
// Read-only view of a finished likelihood's device data (multibin batches)
// ---------------------------------------------------------------------------
struct LikelihoodView {
	const float2* amps;       // tiled store
	uint64_t nEvents;
	uint32_t storeB;
	int W0, W, R, P;
	std::vector<int> slotRe, slotIm;  // host copies, [R*W]
	const double* accI;       // device, reordered acceptance blocks
	double nEvt, totAcc;
	int prior;
	double cauchyWidth;
	int device;
	std::vector<unsigned char> fixed;  // [P] 1 for parameters the layout holds fixed
};
int likelihoodView(const pwa_likelihood* L, LikelihoodView* v);
// One launch of the likelihood's own FdF kernel (its plan, any rank and
// reflectivities) at device parameters dPar into dOut [P + 2] on stream s;
// with dActive non-null the launch returns at once when *dActive == 0.
// Stream-ordered, no synchronisation or allocation (capturable).
int launchLikelihoodEval(pwa_likelihood* L, const double* dPar, double* dOut, const int* dActive, cudaStream_t s);
// clears the likelihood's device error flag (stream-ordered)
int clearLikelihoodError(pwa_likelihood* L, cudaStream_t s);

// ---------------------------------------------------------------------------
// Batched multibin x multistart FdF and L-BFGS (multibin.cu)
// ---------------------------------------------------------------------------
struct BinDesc {
	const float2* amps;  // tiled store of the bin (B = 128)
	uint64_t nEvents;
	const double* accI;  // W x W complex128 acceptance integral (one reflectivity)
	double nEvt, totAcc;
	int q0;              // first problem of the bin
	int nStarts;
};
struct BatchItem {
	int bin, group;      // starts [group * SG, ...) of the bin
	uint32_t t0, t1;     // tiles [t0, t1) of the bin
};
struct ProblemDesc {
	int bin, slot;       // slot within its start group
	int item0, item1;    // items of its (bin, group)
};
struct BatchArgs {
	const BinDesc* bins;
	const BatchItem* items;
	int nItems;
	int W, P, SG;
	const int* slotRe;   // [W] parameter index of Re V_w or -1 (rank 1)
	const int* slotIm;
	const double* x;     // [Q][P] trial points
	const int* active;   // [Q]
	double* partials;    // [nItems][SG][2 + 2W]
	unsigned* devErr;
};
struct FinishBatchArgs {
	const BinDesc* bins;
	const ProblemDesc* problems;
	int Q, W, P, SG;
	const int* slotRe;
	const int* slotIm;
	const double* x;
	const int* active;
	const double* partials;
	int prior;
	double cauchyWidth;
	const unsigned char* fixed;  // [bins][P] parameters held fixed (gradient components set to 0)
	double* f;           // [Q]
	double* g;           // [Q][P]
};
// general-layout batches: f and the gradient of every active problem from
// its FdF launch's output [Q][P + 2] into the L-BFGS buffers, fixed
// parameters' gradient components set to 0, device error flags collected
struct GatherEvalArgs {
	int Q, P;
	const double* out;           // [Q][P + 2]
	const int* active;           // [Q]
	const ProblemDesc* problems; // [Q]
	const unsigned char* fixed;  // [bins][P]
	double* f;                   // [Q]
	double* g;                   // [Q][P]
	unsigned* devErr;
};
int launchGatherEval(const GatherEvalArgs& a, cudaStream_t s);
enum { kLbfgsInit = 0, kLbfgsSearch = 1, kLbfgsConverged = 2, kLbfgsMaxIter = 3, kLbfgsStalled = 4, kLbfgsFailed = 5,
       kLbfgsFloor = 6 };
struct LbfgsArgs {
	int Q, P, m, maxIter;
	int floorWindow;               // iterations without a 1% better gradient norm -> kLbfgsFloor (0: off)
	double gtolAbs, gtolRel;
	double *x, *g, *d, *xt;        // [Q][P]
	const double* ft;              // [Q] trial values
	const double* gt;              // [Q][P] trial gradients
	double *f, *gnorm, *step, *gamma, *gBest;  // [Q]
	double *S, *Y;                 // [Q][m][P]
	double *rho, *alphaBuf;        // [Q][m]
	int *status, *iter, *nBack, *hist, *head, *itBest;  // [Q]
};
size_t batchSmemBytes(int W, int SG);
// sets the kernel's shared-memory limit (before any launch or stream capture)
int configureBatchFdf(int W, int SG, size_t maxSmem);
int launchBatchFdf(const BatchArgs& a, int numSMs, cudaStream_t s);
int launchBatchFinish(const FinishBatchArgs& a, cudaStream_t s);
int launchLbfgs(const LbfgsArgs& a, cudaStream_t s);
int launchCountActive(const int* status, int Q, int* active, unsigned* nActive, cudaStream_t s);

// ---------------------------------------------------------------------------
// Warm-start network kernels (mlp.cu)
// ---------------------------------------------------------------------------
// C[M][N] = sum_k A(m, k) B(k, n) (+ bias[n], relu, relu mask), BF16 operands
// A(m, k) = A[m * lda_m + k * lda_k], B(k, n) = B[k * ldb_k + n * ldb_n]
struct MlpGemm {
	int M, N, K;
	const uint16_t* A;
	size_t lda_m, lda_k;
	int aContigK;        // 1 when lda_k == 1 (load order along k)
	const uint16_t* B;
	size_t ldb_k, ldb_n;
	int bContigK;        // 1 when ldb_k == 1
	const float* bias;   // [N] or null
	int relu;
	const uint16_t* mask;  // BF16 [M][N]: zero the output where mask <= 0, or null
	float* C32;          // FP32 [M][N] or null
	uint16_t* C16;       // BF16 [M][N] or null
	int splitK;          // K slices (whole K steps of 64): FP32 partials in work, then the epilogue kernel
	float* work;         // FP32 [splitK][M][N]
	unsigned* devErr;    // device error flag (a bounded wait of the tensor-core kernel expired)
};
// K slices for the tensor-core GEMM (its blocks cover the SMs about twice)
int mlpGemmSplit(const MlpGemm& g, int numSMs);
int launchMlpGemm(const MlpGemm& g, cudaStream_t s);
int launchColSum(const float* X, int M, int N, float* out, cudaStream_t s);
int launchMse(const float* Y, const float* T, int n, float scale, float* dY32, uint16_t* dY16, double* loss,
              cudaStream_t s);
int launchAdam(float* w, const float* g, float* m, float* v, uint16_t* w16, size_t n, float lr, float b1, float b2,
               float eps, float c1, float c2, cudaStream_t s);
int launchToBf16(const float* x, uint16_t* y, size_t n, cudaStream_t s);
int launchGatherRows(const void* src, const uint32_t* idx, int rows, size_t rowBytes, void* dst, cudaStream_t s);

// ---------------------------------------------------------------------------
// On-the-fly event binning (otf_kernels.cu)
// ---------------------------------------------------------------------------
constexpr int kOtfMaxVars = 8;
constexpr int kOtfChunk = 4096;  // events per block of the selection kernels
struct OtfArgs {
	int nVars;
	double lower[kOtfMaxVars], upper[kOtfMaxVars];
	const double* vars;  // device, [nVars][n]
	uint64_t n;
};
int launchOtfCount(const OtfArgs& a, unsigned* counts, cudaStream_t s);
int launchOtfCompact(const OtfArgs& a, const unsigned long long* offsets, unsigned long long* idx, cudaStream_t s);
int launchOtfGather(const void* src, const unsigned long long* idx, uint64_t n, int elemBytes, void* dst,
                    cudaStream_t s);

// ---------------------------------------------------------------------------
// Raw amplitude files (ampfile.cpp)
// ---------------------------------------------------------------------------
struct AmpFile {
	std::string path;
	int fd = -1;
	uint32_t nWaves = 0, nVars = 0;
	uint64_t nEvents = 0, dataOffset = 0;
	std::vector<std::string> waves, vars;
	AmpFile() = default;
	AmpFile(const AmpFile&) = delete;
	AmpFile& operator=(const AmpFile&) = delete;
	AmpFile(AmpFile&& o) noexcept { *this = std::move(o); }
	AmpFile& operator=(AmpFile&& o) noexcept;
	~AmpFile();
	uint64_t waveOffset(uint32_t w) const { return dataOffset + (uint64_t)w * nEvents * 8; }
	uint64_t varOffset(uint32_t v) const { return dataOffset + ((uint64_t)nWaves + v) * nEvents * 8; }
};
// opens and validates an amplitude file (header, name table, file size)
int ampFileOpen(const char* path, AmpFile& f);
// file bytes [offset, offset + bytes) -> device memory (synchronises s)
int ampFileToDevice(const AmpFile& f, uint64_t offset, uint64_t bytes, void* dst, cudaStream_t s);
// header bytes of an amplitude file up to its data block (names: the waves,
// then the binning variables) and positioned writes into an open file
int ampFileHeader(uint32_t nWaves, uint32_t nVars, const char* const* names, uint64_t nEvents,
                  std::vector<unsigned char>& header);
int ampFilePwrite(int fd, const void* p, size_t bytes, uint64_t offset, const char* path);
// a file written as <path>.tmp and renamed to <path> by commit(), so that a
// failed write never leaves a truncated file with a valid header at <path>;
// without commit() the destructor closes and removes the temporary file
struct AmpFileWriter {
	int fd = -1;
	std::string path, tmp;
	AmpFileWriter() = default;
	AmpFileWriter(const AmpFileWriter&) = delete;
	AmpFileWriter& operator=(const AmpFileWriter&) = delete;
	~AmpFileWriter();
	int create(const char* finalPath);
	int commit();
};

// ---------------------------------------------------------------------------
// Three-body isobar amplitudes (isobar.cu, plan in isobar_plan.h)
// ---------------------------------------------------------------------------
namespace iso {
struct PlanView;
}
// amps complex128 (fp32 false) or complex64 (fp32 true: per-wave arithmetic
// in FP32) [wave][n] from beam [3][n] and final state [3][3][n] (device
// pointers; the view's arrays in device memory)
int launchIsobarAmplitudes(const iso::PlanView& v, const double* beam, const double* fs, uint64_t n, void* amps,
                           bool fp32, cudaStream_t s);

}  // namespace pwa
