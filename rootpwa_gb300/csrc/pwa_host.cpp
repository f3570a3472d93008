// pwa_host.cpp -- host side of the GB300 extended-likelihood engine: the
// C ABI of include/pwa_gb300.h over two C++ objects that mirror ROOTPWA's
// rpwa::ampIntegralMatrix and rpwa::pwaLikelihood<complex<double>>.
//
// Setup (wave list, parameter layout, integral reordering and rescaling,
// amplitude normalisation) follows the reference line by line in FP64 on the
// host; every per-event loop runs in the CUDA kernels of this directory.

#include "../../include/pwa_gb300.h"
#include "pwa_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

typedef std::complex<double> cplx;

namespace {
thread_local std::string g_lastError;
std::atomic<uint64_t> g_launches{0};
}  // namespace

namespace pwa {

int setError(int code, const std::string& msg)
{
	if (code != kOk)
		g_lastError = msg;
	return code;
}

int cudaCheck(cudaError_t e, const char* what)
{
	if (e == cudaSuccess)
		return kOk;
	cudaGetLastError();  // clear the sticky-free error state of the runtime
	return setError(e == cudaErrorMemoryAllocation ? kErrOom : kErrCuda,
	                std::string(what) + ": " + cudaGetErrorString(e));
}

void countLaunches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

// device allocation owned by a handle
// Test hook: after this many further device allocations, every allocation
// fails with PWA_ERROR_OUT_OF_MEMORY before it reaches cudaMalloc (negative:
// off).  Host-side fault injection for the error paths.
std::atomic<long> g_failAllocAfter{-1};

struct DevBuf {
	void* p = nullptr;
	size_t bytes = 0;
	DevBuf() = default;
	DevBuf(const DevBuf&) = delete;
	DevBuf& operator=(const DevBuf&) = delete;
	~DevBuf() { release(); }
	int alloc(size_t b, const char* what)
	{
		release();
		if (b == 0)
			return kOk;
		if (g_failAllocAfter.load() >= 0 && g_failAllocAfter.fetch_sub(1) <= 0) {
			g_failAllocAfter.store(0);
			return setError(kErrOom, std::string(what) + ": injected allocation failure");
		}
		const cudaError_t e = cudaMalloc(&p, b);
		if (e != cudaSuccess) {
			p = nullptr;
			return cudaCheck(e, what);
		}
		bytes = b;
		return kOk;
	}
	int ensure(size_t b, const char* what) { return (bytes >= b && p) ? kOk : alloc(b, what); }
	void release()
	{
		if (p)
			cudaFree(p);
		p = nullptr;
		bytes = 0;
	}
	template <typename T>
	T* as() const
	{
		return static_cast<T*>(p);
	}
};

// page-locked host staging buffer
struct PinnedBuf {
	void* p = nullptr;
	size_t bytes = 0;
	PinnedBuf() = default;
	PinnedBuf(const PinnedBuf&) = delete;
	PinnedBuf& operator=(const PinnedBuf&) = delete;
	~PinnedBuf() { release(); }
	void* dev = nullptr;  // device view of a mapped buffer
	int ensure(size_t b, const char* what, bool mapped = false)
	{
		if (p && bytes >= b && (!mapped || dev))
			return kOk;
		release();
		const cudaError_t e = mapped ? cudaHostAlloc(&p, b, cudaHostAllocMapped) : cudaMallocHost(&p, b);
		if (e != cudaSuccess) {
			p = nullptr;
			return cudaCheck(e, what);
		}
		bytes = b;
		if (mapped) {
			const cudaError_t e2 = cudaHostGetDevicePointer(&dev, p, 0);
			if (e2 != cudaSuccess) {
				release();
				return cudaCheck(e2, what);
			}
		}
		return kOk;
	}
	void release()
	{
		if (p)
			cudaFreeHost(p);
		p = nullptr;
		dev = nullptr;
		bytes = 0;
	}
	template <typename T>
	T* as() const
	{
		return static_cast<T*>(p);
	}
};

#define PWA_TRY(expr)                 \
	do {                              \
		const int _st = (expr);       \
		if (_st != kOk)               \
			return _st;               \
	} while (0)

int deviceInfo(int* dev, int* sms, size_t* smem)
{
	PWA_TRY(cudaCheck(cudaGetDevice(dev), "cudaGetDevice"));
	PWA_TRY(cudaCheck(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, *dev), "SM count"));
	int optin = 0;
	PWA_TRY(cudaCheck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, *dev), "smem"));
	*smem = (size_t)optin;
	return kOk;
}

std::string fmtDouble(double v)
{
	char buf[64];
	std::snprintf(buf, sizeof(buf), "%.16e", v);
	return buf;
}

}  // namespace
}  // namespace pwa

using namespace pwa;

// ===========================================================================
// ampIntegralMatrix
// ===========================================================================
struct pwa_integral {
	uint32_t nWaves = 0;
	uint64_t nEvents = 0;
	std::vector<std::string> names;
	std::vector<cplx> sums;  // raw sums [i][j]

	int index(const std::string& n) const
	{
		for (size_t i = 0; i < names.size(); ++i)
			if (names[i] == n)
				return (int)i;
		return -1;
	}
	bool sameWaveSet(const pwa_integral& o) const
	{
		if (o.nWaves != nWaves)
			return false;
		for (const auto& n : names)
			if (o.index(n) < 0)
				return false;
		return true;
	}
};

namespace {

// Sums the GPU Gram kernel for integrate().
int gramOnDevice(uint32_t W, const void* amps, uint64_t nEvents, uint32_t nSub, int ampType, int memory,
                 const std::vector<double>& weightK, uint64_t K, int precision, std::vector<cplx>& out)
{
	int dev, sms;
	size_t smem;
	PWA_TRY(deviceInfo(&dev, &sms, &smem));
	cudaStream_t s = nullptr;
	PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream"));
	struct StreamGuard {
		cudaStream_t s;
		~StreamGuard() { cudaStreamDestroy(s); }
	} guard{s};

	// device inputs may still be written by the caller's streams
	if (memory == PWA_MEMORY_DEVICE)
		PWA_TRY(cudaCheck(cudaDeviceSynchronize(), "synchronise before reading device amplitudes"));
	const uint64_t ldIn = nEvents * nSub;
	const bool wantDouble = (precision == PWA_PRECISION_FP64 && ampType == PWA_COMPLEX128);
	const bool tensorCore = (precision == PWA_PRECISION_TF32 || precision == PWA_PRECISION_TF32X3 ||
	                         precision == PWA_PRECISION_BF16X3);
	// the tensor-core kernel reads rows with TMA: even row stride (16-byte
	// multiple) and a 16-byte aligned base
	const uint64_t ldPad = tensorCore ? (K + (K & 1ull)) : K;
	DevBuf dIn, dConv, dW, dPart, dOut, dErr;
	const float2* a32 = nullptr;
	const double2* a64 = nullptr;
	uint64_t ldK = ldIn;
	if (memory == PWA_MEMORY_DEVICE) {
		if (ampType == PWA_COMPLEX64) {
			a32 = static_cast<const float2*>(amps);
			if (tensorCore && ((ldIn & 1ull) || (reinterpret_cast<uintptr_t>(amps) & 15u))) {
				PWA_TRY(dConv.alloc((size_t)W * ldPad * sizeof(float2), "integral alignment buffer"));
				PWA_TRY(cudaCheck(cudaMemcpy2DAsync(dConv.p, ldPad * sizeof(float2), amps, ldIn * sizeof(float2),
				                                    K * sizeof(float2), W, cudaMemcpyDeviceToDevice, s),
				                  "integral amplitude realignment"));
				a32 = dConv.as<float2>();
				ldK = ldPad;
			}
		} else if (wantDouble) {
			a64 = static_cast<const double2*>(amps);
		} else {
			PWA_TRY(dConv.alloc((size_t)W * ldPad * sizeof(float2), "integral conversion buffer"));
			PWA_TRY(dErr.alloc(sizeof(unsigned), "flag"));
			for (uint32_t w = 0; w < W; ++w)
				PWA_TRY(launchConvertPlain(static_cast<const double2*>(amps) + (size_t)w * ldIn,
				                           dConv.as<float2>() + (size_t)w * ldPad, K, s));
			a32 = dConv.as<float2>();
			ldK = ldPad;
		}
	} else {
		const size_t elem = (ampType == PWA_COMPLEX64) ? sizeof(float2) : sizeof(double2);
		PWA_TRY(dIn.alloc((size_t)W * ldPad * elem, "integral amplitude buffer"));
		PWA_TRY(cudaCheck(cudaMemcpy2DAsync(dIn.p, ldPad * elem, amps, ldIn * elem, K * elem, W,
		                                    cudaMemcpyHostToDevice, s),
		                  "integral amplitude upload"));
		ldK = ldPad;
		if (ampType == PWA_COMPLEX64) {
			a32 = dIn.as<float2>();
		} else if (wantDouble) {
			a64 = dIn.as<double2>();
		} else {
			PWA_TRY(dConv.alloc((size_t)W * ldPad * sizeof(float2), "integral conversion buffer"));
			PWA_TRY(dErr.alloc(sizeof(unsigned), "flag"));
			PWA_TRY(launchConvertPlain(dIn.as<double2>(), dConv.as<float2>(), (uint64_t)W * ldPad, s));
			a32 = dConv.as<float2>();
		}
	}
	if (!weightK.empty()) {
		// the tensor-core kernel weights both operands by sqrt(w)
		if (tensorCore)
			for (double v : weightK)
				if (!(v >= 0.))
					return setError(kErrUnsupported, "tensor-core Gram needs non-negative event weights");
		PWA_TRY(dW.alloc(weightK.size() * sizeof(double), "weights"));
		PWA_TRY(cudaCheck(cudaMemcpyAsync(dW.p, weightK.data(), weightK.size() * sizeof(double),
		                                  cudaMemcpyHostToDevice, s),
		                  "weight upload"));
	}
	PWA_TRY(dOut.alloc((size_t)W * W * 2 * sizeof(double), "integral output"));
	if (!dErr.p)
		PWA_TRY(dErr.alloc(sizeof(unsigned), "flag"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dErr.p, 0, sizeof(unsigned), s), "memset"));

	GramArgs g{};
	g.amps = a32;
	g.amps64 = a64;
	g.K = K;
	g.ldK = ldK;
	g.W = (int)W;
	g.weightK = weightK.empty() ? nullptr : dW.as<double>();
	g.devErr = dErr.as<unsigned>();
	int st = kErrUnsupported;
	if (tensorCore) {
		const size_t scratch = gramTcScratchFloats((int)W, sms) / 2 + 1;  // doubles holding the FP32 partials
		PWA_TRY(dPart.alloc(scratch * sizeof(double), "gram partials"));
		st = launchGramTc(g, precision, sms, s, dOut.as<double>(), dPart.as<double>(), scratch);
		if (st != kOk)
			return st;
	} else {
		const int tps = ((int)W + 63) / 64;
		const int nTiles = tps * (tps + 1) / 2;
		int chunks = std::max(1, (4 * sms + nTiles - 1) / nTiles);
		const uint64_t maxChunks = std::max<uint64_t>(1, K / 64);
		chunks = (int)std::min<uint64_t>((uint64_t)chunks, maxChunks);
		g.chunks = chunks;
		PWA_TRY(dPart.alloc((size_t)chunks * W * W * 2 * sizeof(double), "gram partials"));
		PWA_TRY(cudaCheck(cudaMemsetAsync(dPart.p, 0, dPart.bytes, s), "memset"));
		g.partials = dPart.as<double>();
		PWA_TRY(launchGramSimt(g, precision, s));
		PWA_TRY(launchGramReduce(g.partials, chunks, (int)W, dOut.as<double>(), 0, s));
	}
	std::vector<double> host((size_t)W * W * 2);
	unsigned devErr = 0;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(host.data(), dOut.p, host.size() * sizeof(double), cudaMemcpyDeviceToHost, s),
	                  "integral download"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(&devErr, dErr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "flag download"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "integral sync"));
	if (devErr)
		return setError(kErrTimeout, "integral kernel: a bounded device-side wait expired");
	out.resize((size_t)W * W);
	for (size_t k = 0; k < out.size(); ++k)
		out[k] = cplx(host[2 * k], host[2 * k + 1]);
	return kOk;
}

}  // namespace

extern "C" {

int pwa_abi_version(void) { return PWA_GB300_ABI_VERSION; }
const char* pwa_last_error(void) { return g_lastError.c_str(); }
uint64_t pwa_kernel_launch_count(void) { return g_launches.load(); }

int pwa_integral_create(pwa_integral** out)
{
	if (!out)
		return setError(kErrArg, "null output pointer");
	try {
		*out = new pwa_integral();
	} catch (const std::bad_alloc&) {
		return setError(kErrOom, "host allocation failed");
	}
	return kOk;
}

int pwa_integral_destroy(pwa_integral* I)
{
	delete I;
	return kOk;
}

int pwa_integral_copy(pwa_integral* dst, const pwa_integral* src)
{
	if (!dst || !src)
		return setError(kErrArg, "null integral");
	if (dst != src)
		*dst = *src;
	return kOk;
}

int pwa_integral_set_wave_names(pwa_integral* I, uint32_t n, const char* const* names)
{
	if (!I || (!names && n))
		return setError(kErrArg, "null argument");
	if (I->nWaves > 0) {
		if (n != I->nWaves)
			return setError(kErrState, "integral matrix was already initialized with a different number of waves");
		for (uint32_t i = 0; i < n; ++i)
			if (I->names[i] != names[i])
				return setError(kErrState, "integral matrix was already initialized with different wave names");
		return kOk;
	}
	I->names.assign(names, names + n);
	I->nWaves = n;
	I->sums.assign((size_t)n * n, cplx(0, 0));
	return kOk;
}

int pwa_integral_integrate(pwa_integral* I, uint32_t nWaves, const char* const* waveNames, const void* amps,
                           uint64_t nEvents, uint32_t nSubAmps, int ampType, int memory, const double* weights,
                           uint64_t nWeights, const uint8_t* inBin, int64_t maxNmbEvents, int precision)
{
	if (!I || !waveNames || !amps)
		return setError(kErrArg, "null argument");
	if (nWaves == 0)
		return setError(kErrArg, "did not receive any amplitudes; cannot calculate integral");
	if (nEvents == 0)
		return setError(kErrArg, "amplitudes contain no values; cannot calculate integral");
	if (nSubAmps == 0)
		return setError(kErrArg, "amplitude object does not contain any amplitude values");
	if (ampType != PWA_COMPLEX64 && ampType != PWA_COMPLEX128)
		return setError(kErrArg, "unknown amplitude type");
	if (memory != PWA_MEMORY_HOST && memory != PWA_MEMORY_DEVICE)
		return setError(kErrArg, "unknown memory kind");
	if (precision < PWA_PRECISION_FP64 || precision > PWA_PRECISION_BF16X3)
		return setError(kErrArg, "unknown precision");
	// wave-name bookkeeping as ampIntegralMatrix.cc:310-330
	if (I->names.empty()) {
		I->names.assign(waveNames, waveNames + nWaves);
		I->nWaves = nWaves;
	} else {
		if (I->names.size() != nWaves)
			return setError(kErrState, "integral matrix was already initialized with a different number of waves");
		for (uint32_t i = 0; i < nWaves; ++i)
			if (I->names[i] != waveNames[i])
				return setError(kErrState, "integral matrix was already initialized with different wave names");
	}
	const uint64_t nProc = (maxNmbEvents <= 0) ? nEvents : std::min<uint64_t>(nEvents, (uint64_t)maxNmbEvents);
	// event selection and weights (ampIntegralMatrix.cc:408-429): the weight
	// stream is consumed by events that pass the bin cut, in order
	std::vector<double> weightK;
	uint64_t counter = 0, wIdx = 0, lastK = nProc;
	bool success = true;
	double wsum = 0., wcomp = 0.;  // compensated sum of 1/w
	const bool useWeight = (weights != nullptr);
	if (useWeight || inBin) {
		weightK.assign(nProc * nSubAmps, 0.);
		for (uint64_t ev = 0; ev < nProc; ++ev) {
			if (inBin && !inBin[ev])
				continue;
			++counter;
			double w = 1.;
			if (useWeight) {
				if (wIdx >= nWeights) {
					success = false;
					lastK = ev;
					break;
				}
				w = weights[wIdx++];
			}
			const double weight = 1. / w;
			const double y = weight - wcomp, t = wsum + y;
			wcomp = (t - wsum) - y;
			wsum = t;
			for (uint32_t s = 0; s < nSubAmps; ++s)
				weightK[ev * nSubAmps + s] = useWeight ? weight : 1.;
		}
	} else {
		counter = nProc;
		wsum = (double)nProc;
	}
	const uint64_t K = nProc * nSubAmps;
	std::vector<cplx> result;
	if (lastK > 0 && counter > 0)
		PWA_TRY(gramOnDevice(nWaves, amps, nEvents, nSubAmps, ampType, memory, weightK, K, precision, result));
	else
		result.assign((size_t)nWaves * nWaves, cplx(0, 0));
	I->nEvents = counter;
	I->sums = result;
	if (useWeight && counter > 0) {
		const double weightNorm = wsum / (double)counter;
		for (auto& v : I->sums)
			v *= 1. / weightNorm;
	}
	if (!success)
		return setError(kErrIo, "weight stream shorter than the number of selected events; integration stopped");
	return kOk;
}

int pwa_integral_add_event(pwa_integral* I, const double* amps)
{
	if (!I || !amps)
		return setError(kErrArg, "null argument");
	const uint32_t n = I->nWaves;
	for (uint32_t i = 0; i < n; ++i) {
		const cplx a(amps[2 * i], amps[2 * i + 1]);
		for (uint32_t j = 0; j < n; ++j)
			I->sums[(size_t)i * n + j] += a * std::conj(cplx(amps[2 * j], amps[2 * j + 1]));
	}
	++I->nEvents;
	return kOk;
}

int pwa_integral_element(const pwa_integral* I, uint32_t i, uint32_t j, double* re, double* im)
{
	if (!I || !re || !im)
		return setError(kErrArg, "null argument");
	if (i >= I->nWaves || j >= I->nWaves)
		return setError(kErrArg, "wave index out of range");
	const cplx v = I->sums[(size_t)i * I->nWaves + j] / (double)I->nEvents;
	*re = v.real();
	*im = v.imag();
	return kOk;
}

int pwa_integral_matrix(const pwa_integral* I, double* out)
{
	if (!I || !out)
		return setError(kErrArg, "null argument");
	for (size_t k = 0; k < I->sums.size(); ++k) {
		out[2 * k] = I->sums[k].real();
		out[2 * k + 1] = I->sums[k].imag();
	}
	return kOk;
}

int pwa_integral_set_matrix(pwa_integral* I, const double* in)
{
	if (!I || !in)
		return setError(kErrArg, "null argument");
	for (size_t k = 0; k < I->sums.size(); ++k)
		I->sums[k] = cplx(in[2 * k], in[2 * k + 1]);
	return kOk;
}

int pwa_integral_nmb_waves(const pwa_integral* I, uint32_t* n)
{
	if (!I || !n)
		return setError(kErrArg, "null argument");
	*n = I->nWaves;
	return kOk;
}

int pwa_integral_nmb_events(const pwa_integral* I, uint64_t* n)
{
	if (!I || !n)
		return setError(kErrArg, "null argument");
	*n = I->nEvents;
	return kOk;
}

int pwa_integral_set_nmb_events(pwa_integral* I, uint64_t n)
{
	if (!I)
		return setError(kErrArg, "null argument");
	I->nEvents = n;
	return kOk;
}

int pwa_integral_wave_name(const pwa_integral* I, uint32_t i, char* buf, uint32_t len)
{
	if (!I || !buf || len == 0)
		return setError(kErrArg, "null argument");
	if (i >= I->names.size())
		return setError(kErrArg, "wave index out of range");
	std::snprintf(buf, len, "%s", I->names[i].c_str());
	return kOk;
}

int pwa_integral_wave_index(const pwa_integral* I, const char* name, uint32_t* index)
{
	if (!I || !name || !index)
		return setError(kErrArg, "null argument");
	const int k = I->index(name);
	if (k < 0)
		return setError(kErrArg, std::string("cannot find wave '") + name + "' in integral matrix");
	*index = (uint32_t)k;
	return kOk;
}

static int integralCombine(pwa_integral* I, const pwa_integral* o, double sign)
{
	if (!I || !o)
		return setError(kErrArg, "null argument");
	if (!I->sameWaveSet(*o))
		return setError(kErrArg, "the two integral matrices have different wave sets");
	const uint32_t n = I->nWaves;
	for (uint32_t i = 0; i < n; ++i) {
		const int oi = o->index(I->names[i]);
		for (uint32_t j = 0; j < n; ++j) {
			const int oj = o->index(I->names[j]);
			I->sums[(size_t)i * n + j] += sign * o->sums[(size_t)oi * n + oj];
		}
	}
	if (sign > 0)
		I->nEvents += o->nEvents;
	else
		I->nEvents -= o->nEvents;
	return kOk;
}

int pwa_integral_add(pwa_integral* I, const pwa_integral* o) { return integralCombine(I, o, 1.); }
int pwa_integral_subtract(pwa_integral* I, const pwa_integral* o) { return integralCombine(I, o, -1.); }

int pwa_integral_scale(pwa_integral* I, double f)
{
	if (!I)
		return setError(kErrArg, "null argument");
	for (auto& v : I->sums)
		v *= f;
	I->nEvents = (uint64_t)((double)I->nEvents * f);
	return kOk;
}

int pwa_integral_divide(pwa_integral* I, double f)
{
	if (!I)
		return setError(kErrArg, "null argument");
	for (auto& v : I->sums)
		v /= f;
	I->nEvents = (uint64_t)((double)I->nEvents / f);
	return kOk;
}

int pwa_integral_renormalize(pwa_integral* I, uint64_t n)
{
	if (!I)
		return setError(kErrArg, "null argument");
	if (I->nEvents == 0)
		return setError(kErrState, "integral has no events");
	PWA_TRY(pwa_integral_scale(I, (double)n / (double)I->nEvents));
	I->nEvents = n;
	return kOk;
}

int pwa_integral_read_ascii(pwa_integral* I, const char* path)
{
	if (!I || !path)
		return setError(kErrArg, "null argument");
	std::ifstream in(path);
	if (!in)
		return setError(kErrIo, std::string("cannot open file '") + path + "' for reading of integral matrix");
	uint32_t nw;
	uint64_t ne;
	if (!(in >> nw >> ne))
		return setError(kErrIo, "could not read number of waves and events");
	uint32_t nr, nc;
	if (!(in >> nr >> nc))
		return setError(kErrIo, "could not read number of rows and columns");
	std::vector<cplx> m((size_t)nr * nc);
	for (uint32_t i = 0; i < nr; ++i)
		for (uint32_t j = 0; j < nc; ++j)
			if (!(in >> m[(size_t)i * nc + j]) || in.eof())
				return setError(kErrIo, "could not read integral values; stream seems truncated");
	uint32_t mapSize;
	in >> mapSize;
	if (mapSize != nw)
		return setError(kErrIo, "mismatch between integral dimensions and number of wave names");
	std::vector<std::string> names(nw);
	while (mapSize > 0 && in) {
		std::string name;
		uint32_t idx;
		if (!(in >> name >> idx))
			return setError(kErrIo, "could not read wave name -> index map; stream seems truncated");
		if (idx >= nw)
			return setError(kErrIo, "wave index out of range in wave name -> index map");
		names[idx] = name;
		--mapSize;
	}
	I->nWaves = nw;
	I->nEvents = ne;
	I->sums = m;
	I->names = names;
	return kOk;
}

int pwa_integral_write_ascii(const pwa_integral* I, const char* path)
{
	if (!I || !path)
		return setError(kErrArg, "null argument");
	std::ofstream out(path);
	if (!out)
		return setError(kErrIo, std::string("cannot open file '") + path + "' for writing of integral matrix");
	out << I->nWaves << "\n" << I->nEvents << "\n" << I->nWaves << " " << I->nWaves << "\n";
	for (uint32_t i = 0; i < I->nWaves; ++i) {
		for (uint32_t j = 0; j < I->nWaves; ++j) {
			const cplx& v = I->sums[(size_t)i * I->nWaves + j];
			out << "(" << fmtDouble(v.real()) << "," << fmtDouble(v.imag()) << ")\t";
		}
		out << "\n";
	}
	out << I->names.size() << "\n";
	for (uint32_t i = 0; i < I->nWaves; ++i)
		out << I->names[i] << " " << i << "\n";
	return out.good() ? kOk : setError(kErrIo, "problems writing integral to ASCII file");
}

}  // extern "C"

// ===========================================================================
// pwaLikelihood
// ===========================================================================
namespace {

struct ParInfo {
	std::string waveName;
	int rank = 0;
	double threshold = 0.;
	bool fixed = false;
	bool realPart = true;
};

struct CallInfo {
	uint64_t nCalls = 0;
	double total = 0., func = 0., norm = 0.;
};

double seconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct pwa_likelihood {
	int device = 0, numSMs = 0;
	size_t maxSmem = 0;
	cudaStream_t stream = nullptr;
	bool ownStream = false;
	bool streamSet = false;  // the caller chose the stream (possibly the default stream)

	bool useNormalizedAmps = true;
	int priorType = PWA_PRIOR_FLAT;
	// event shard (pwa_likelihood_set_shard): only the root shard adds the
	// normalisation and prior terms, with the total event count
	bool shardSet = false, shardRoot = true;
	uint64_t shardTotal = 0;
	double cauchyWidth = 0.5;
	int reduction = PWA_REDUCE_FP64;

	uint32_t nW[2] = {0, 0}, nWmax = 0, rank = 1;
	std::vector<std::string> names[2];
	std::vector<double> thres[2];
	std::map<std::string, std::pair<uint32_t, uint32_t> > waveIdx;

	uint32_t nPars = 0;
	std::vector<ParInfo> pars;
	std::vector<int> slotRe, slotIm;  // [rank][W], global wave order (negative first)

	std::vector<cplx> normM, accM;  // [2][nWmax][2][nWmax]
	uint64_t numbAccEvents = 0;
	double totAcc = 0.;
	std::vector<double> psInt;

	uint64_t nEvents = 0;
	uint32_t storeB = 128;  // events per store block (storeIndex)
	// on-the-fly binning: indices of the selected events of the data file
	bool otfSet = false;
	uint64_t otfFileEvents = 0, otfSelected = 0;
	DevBuf otfIdx;
	DevBuf amps, ampTmp;
	std::vector<char> added[2];

	bool initialized = false, normAdded = false, accAdded = false, finished = false;

	// evaluation resources
	bool autotune = true;
	FdfPlan plan;
	DevBuf dSlotRe, dSlotIm, dAccI, dFixAcc, dNfAcc, dCounter, dErr, dPar, dOut, dFlag;
	PinnedBuf hPar, hOut;
	cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};

	std::vector<double> parCache, derivCache;
	bool cacheValid = false;
	CallInfo info[5];

	// per-evaluation kernel timing (pwa_likelihood_set_timing)
	bool timing = false;
	std::vector<cudaEvent_t> timingEvents;  // 3 per evaluation
	size_t nTimed = 0;

	uint32_t W() const { return nW[0] + nW[1]; }
	uint32_t gw(uint32_t e, uint32_t w) const { return e == 0 ? w : nW[0] + w; }
	size_t mIdx(uint32_t e1, uint32_t i, uint32_t e2, uint32_t j) const
	{
		return (((size_t)e1 * nWmax + i) * 2 + e2) * nWmax + j;
	}

	~pwa_likelihood()
	{
		for (auto& e : ev)
			if (e)
				cudaEventDestroy(e);
		for (auto& e : timingEvents)
			cudaEventDestroy(e);
		if (ownStream && stream)
			cudaStreamDestroy(stream);
	}
};

namespace {

int checkFinished(const pwa_likelihood* L)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (!L->finished)
		return setError(kErrState, "pwaLikelihood::finishInit has not been called");
	return kOk;
}

// nEvt of the normalisation term (pwaLikelihood.cc:257): 1 with normalised
// amplitudes, else the number of data events; zero on non-root shards
double normFactor(const pwa_likelihood* L)
{
	if (L->shardSet && !L->shardRoot)
		return 0.;
	if (L->useNormalizedAmps)
		return 1.;
	return (double)(L->shardSet ? L->shardTotal : L->nEvents);
}

int priorOf(const pwa_likelihood* L) { return (L->shardSet && !L->shardRoot) ? PWA_PRIOR_FLAT : L->priorType; }

// Binds the handle to the current CUDA device on first device use (setup of
// the wave set and parameter layout is pure host work).
int ensureDevice(pwa_likelihood* L)
{
	if (L->numSMs > 0)
		return kOk;
	PWA_TRY(deviceInfo(&L->device, &L->numSMs, &L->maxSmem));
	if (!L->streamSet) {
		PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "stream create"));
		L->ownStream = true;
		L->streamSet = true;
	}
	for (auto& e : L->ev)
		if (!e)
			PWA_TRY(cudaCheck(cudaEventCreate(&e), "event create"));
	return kOk;
}

// copyFromParArray (pwaLikelihood.cc:1682-1710), host FP64
void fromPar(const pwa_likelihood* L, const double* par, std::vector<cplx>& V, double& flat)
{
	const uint32_t W = L->W();
	V.assign((size_t)L->rank * W, cplx(0, 0));
	for (uint32_t r = 0; r < L->rank; ++r)
		for (uint32_t g = 0; g < W; ++g) {
			const int ir = L->slotRe[r * W + g], ii = L->slotIm[r * W + g];
			V[(size_t)r * W + g] = cplx(ir >= 0 ? par[ir] : 0., ii >= 0 ? par[ii] : 0.);
		}
	flat = par[L->nPars - 1];
}

// copyToParArray (pwaLikelihood.cc:1716-1731)
void toPar(const pwa_likelihood* L, const std::vector<cplx>& V, double flat, double* out)
{
	const uint32_t W = L->W();
	for (uint32_t r = 0; r < L->rank; ++r)
		for (uint32_t g = 0; g < W; ++g) {
			const int ir = L->slotRe[r * W + g], ii = L->slotIm[r * W + g];
			if (ir >= 0)
				out[ir] = V[(size_t)r * W + g].real();
			if (ii >= 0)
				out[ii] = V[(size_t)r * W + g].imag();
		}
	out[L->nPars - 1] = flat;
}

// Launches the fused FdF kernel: dPar -> dOut (f, gradient, device status).
int launchEval(pwa_likelihood* L, const double* dPar, double* dOut, int withGrad, cudaStream_t s,
               cudaEvent_t after = nullptr)
{
	FdfArgs a{};
	a.amps = L->amps.as<float2>();
	a.nEvents = L->nEvents;
	a.W0 = (int)L->nW[0];
	a.W = (int)L->W();
	a.R = (int)L->rank;
	a.P = (int)L->nPars;
	a.par = dPar;
	a.slotRe = L->dSlotRe.as<int>();
	a.slotIm = L->dSlotIm.as<int>();
	a.accI = L->dAccI.as<double>();
	a.nEvt = normFactor(L);
	a.totAcc = L->totAcc;
	a.prior = priorOf(L);
	a.cauchyWidth = L->cauchyWidth;
	a.withGrad = withGrad;
	a.reduction = L->reduction;
	a.nPartial = 2 + 2 * a.R * a.W;
	a.fixAcc = L->dFixAcc.as<unsigned long long>();
	a.nfAcc = L->dNfAcc.as<double>();
	a.counter = L->dCounter.as<unsigned>();
	a.devErr = L->dErr.as<unsigned>();
	a.out = dOut;
	cudaEvent_t* te = nullptr;
	if (L->timing && 2 * (L->nTimed + 1) <= L->timingEvents.size()) {
		te = &L->timingEvents[2 * L->nTimed];
		++L->nTimed;
		cudaEventRecord(te[0], s);
	}
	PWA_TRY(launchFdf(L->plan, a, s));
	if (after)
		cudaEventRecord(after, s);
	if (te)
		cudaEventRecord(te[1], s);
	return kOk;
}

// Host-buffer evaluation: par (host) -> f, grad (host).
int hostEval(pwa_likelihood* L, const double* par, double* f, double* grad, int withGrad, int call)
{
	PWA_TRY(checkFinished(L));
	const double t0 = seconds();
	const uint32_t P = L->nPars;
	// the kernel reads the parameters from and writes the results to mapped
	// pinned host memory: one launch and one synchronisation per call, no
	// separate copies (a previous call's kernel has finished: it was waited for)
	PWA_TRY(L->hPar.ensure(P * sizeof(double), "pinned parameters", true));
	PWA_TRY(L->hOut.ensure((P + 2) * sizeof(double), "pinned result", true));
	std::memcpy(L->hPar.as<double>(), par, P * sizeof(double));
	cudaStream_t s = L->stream;
	cudaEventRecord(L->ev[0], s);
	PWA_TRY(launchEval(L, static_cast<const double*>(L->hPar.dev), static_cast<double*>(L->hOut.dev), withGrad, s,
	                   L->ev[1]));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "FdF sync"));
	const double* out = L->hOut.as<double>();
	if (out[P + 1] != 0.) {
		const unsigned flags = (unsigned)out[P + 1];
		cudaMemsetAsync(L->dErr.p, 0, sizeof(unsigned), s);
		cudaStreamSynchronize(s);
		if (flags & kDevErrBounds)
			return setError(kErrNumerical, "debug build: a shared-memory access of the FdF kernel failed its bounds check");
		return setError(kErrTimeout, "a bounded device-side wait expired in the FdF kernel");
	}
	if (f)
		*f = out[0];
	if (withGrad && grad)
		std::memcpy(grad, out + 1, P * sizeof(double));
	if (withGrad) {
		L->parCache.assign(par, par + P);
		L->derivCache.assign(out + 1, out + 1 + P);
		L->cacheValid = true;
	}
	float ms1 = 0.f;
	cudaEventElapsedTime(&ms1, L->ev[0], L->ev[1]);
	CallInfo& ci = L->info[call];
	++ci.nCalls;
	ci.func += ms1 * 1e-3;  // the fused kernel includes the normalisation term
	ci.total += seconds() - t0;
	return kOk;
}

}  // namespace

namespace {

// Plans chosen by the autotuner, per (waves, negative waves, rank, event-count
// class) in this process.
struct TuneKey {
	uint32_t W, W0, R, evClass;
	bool operator<(const TuneKey& o) const
	{
		return std::tie(W, W0, R, evClass) < std::tie(o.W, o.W0, o.R, o.evClass);
	}
};
std::map<TuneKey, std::pair<int, int> > g_tuned;  // -> (pipeline stages, kernel variant)
std::mutex g_tunedMutex;

bool tunedLookup(const TuneKey& key, std::pair<int, int>* v)
{
	std::lock_guard<std::mutex> lock(g_tunedMutex);
	auto it = g_tuned.find(key);
	if (it == g_tuned.end())
		return false;
	*v = it->second;
	return true;
}

void tunedStore(const TuneKey& key, std::pair<int, int> v)
{
	std::lock_guard<std::mutex> lock(g_tunedMutex);
	g_tuned[key] = v;
}

// name of the current CUDA device, empty without one
std::string deviceName()
{
	int dev = 0;
	cudaDeviceProp prop;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
		cudaGetLastError();
		return std::string();
	}
	return std::string(prop.name);
}

// Times every candidate (tile size, pipeline depth) on the handle's own data
// with a fixed parameter point and keeps the fastest.
int autotunePlan(pwa_likelihood* L, const std::vector<FdfPlan>& cands)
{
	uint32_t evClass = 0;
	for (uint64_t n = L->nEvents; n > 1; n >>= 1)
		++evClass;
	const TuneKey key{L->W(), L->nW[0], L->rank, evClass};
	std::pair<int, int> known;
	if (tunedLookup(key, &known)) {
		for (const auto& c : cands)
			if (c.stages == known.first && c.phase1Events == known.second)
				L->plan = c;
		return kOk;
	}
	cudaStream_t s = L->stream;
	std::vector<double> p(L->nPars, 0.5);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(L->dPar.p, p.data(), p.size() * sizeof(double), cudaMemcpyHostToDevice, s),
	                  "autotune parameters"));
	// three rounds over the candidates (so that clock and cache transients
	// do not favour the first), the fastest round of each candidate counts
	std::vector<float> best(cands.size(), 1e30f);
	for (int round = 0; round < 3; ++round)
		for (size_t ci = 0; ci < cands.size(); ++ci) {
			L->plan = cands[ci];
			for (int i = 0; i < 2; ++i)
				PWA_TRY(launchEval(L, L->dPar.as<double>(), L->dOut.as<double>(), 1, s));
			PWA_TRY(cudaCheck(cudaEventRecord(L->ev[0], s), "event"));
			for (int i = 0; i < 8; ++i)
				PWA_TRY(launchEval(L, L->dPar.as<double>(), L->dOut.as<double>(), 1, s));
			PWA_TRY(cudaCheck(cudaEventRecord(L->ev[1], s), "event"));
			PWA_TRY(cudaCheck(cudaEventSynchronize(L->ev[1]), "autotune sync"));
			float ms = 0.f;
			PWA_TRY(cudaCheck(cudaEventElapsedTime(&ms, L->ev[0], L->ev[1]), "elapsed"));
			best[ci] = std::min(best[ci], ms);
		}
	FdfPlan bestPlan = cands.front();
	float bestMs = 1e30f;
	for (size_t ci = 0; ci < cands.size(); ++ci)
		if (best[ci] < bestMs) {
			bestMs = best[ci];
			bestPlan = cands[ci];
		}
	L->plan = bestPlan;
	tunedStore(key, std::make_pair(bestPlan.stages, bestPlan.phase1Events));
	// the tuning runs leave no device error behind
	unsigned err = 0;
	PWA_TRY(cudaCheck(cudaMemcpy(&err, L->dErr.p, sizeof(unsigned), cudaMemcpyDeviceToHost), "error flag"));
	if (err != 0)
		return setError(kErrTimeout, "a bounded device-side wait expired while tuning the FdF kernel");
	return kOk;
}

}  // namespace

extern "C" {

int pwa_likelihood_create(pwa_likelihood** out)
{
	if (!out)
		return setError(kErrArg, "null output pointer");
	try {
		*out = new pwa_likelihood();
	} catch (const std::bad_alloc&) {
		return setError(kErrOom, "host allocation failed");
	}
	return kOk;
}

int pwa_likelihood_destroy(pwa_likelihood* L)
{
	if (L) {
		if (L->stream)
			cudaStreamSynchronize(L->stream);
		delete L;
	}
	return kOk;
}

int pwa_likelihood_use_normalized_amps(pwa_likelihood* L, int flag)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	L->useNormalizedAmps = flag != 0;
	return kOk;
}

int pwa_likelihood_set_prior_type(pwa_likelihood* L, int p)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (p != PWA_PRIOR_FLAT && p != PWA_PRIOR_HALF_CAUCHY)
		return setError(kErrArg, "unknown prior type");
	L->priorType = p;
	return kOk;
}

int pwa_likelihood_set_cauchy_width(pwa_likelihood* L, double w)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	L->cauchyWidth = w;
	return kOk;
}

int pwa_likelihood_set_otf_binning(pwa_likelihood* L, uint32_t nVars, const double* lower, const double* upper,
                                   const double* const* binVars, uint64_t nFileEvents, int memory)
{
	if (!L || (nVars && (!lower || !upper || !binVars)))
		return setError(kErrArg, "null argument");
	if (!L->initialized)
		return setError(kErrState, "likelihood not initialized");
	if (L->finished || L->nEvents != 0)
		return setError(kErrState, "setOnTheFlyBinning must come before addAmplitude()");
	if (nVars > (uint32_t)kOtfMaxVars)
		return setError(kErrArg, "at most 8 binning variables");
	if (nFileEvents == 0)
		return setError(kErrArg, "no events in the data file");
	if (memory != PWA_MEMORY_HOST && memory != PWA_MEMORY_DEVICE)
		return setError(kErrArg, "unknown memory kind");
	PWA_TRY(ensureDevice(L));
	cudaStream_t s = L->stream;
	OtfArgs a{};
	a.nVars = (int)nVars;
	a.n = nFileEvents;
	for (uint32_t v = 0; v < nVars; ++v) {
		a.lower[v] = lower[v];
		a.upper[v] = upper[v];
	}
	DevBuf vars, counts, offsets;
	PWA_TRY(vars.alloc(std::max<uint64_t>(1, nVars) * nFileEvents * sizeof(double), "binning variables"));
	if (memory == PWA_MEMORY_DEVICE)
		PWA_TRY(cudaCheck(cudaDeviceSynchronize(), "synchronise before reading device binning variables"));
	for (uint32_t v = 0; v < nVars; ++v)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(vars.as<double>() + (size_t)v * nFileEvents, binVars[v],
		                                  nFileEvents * sizeof(double),
		                                  memory == PWA_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
		                                  s),
		                  "binning variable upload"));
	a.vars = vars.as<double>();
	const uint64_t blocks = (nFileEvents + kOtfChunk - 1) / kOtfChunk;
	PWA_TRY(counts.alloc(blocks * sizeof(unsigned), "OTF counts"));
	PWA_TRY(launchOtfCount(a, counts.as<unsigned>(), s));
	std::vector<unsigned> hc(blocks);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(hc.data(), counts.p, blocks * sizeof(unsigned), cudaMemcpyDeviceToHost, s),
	                  "OTF counts"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "OTF counts"));
	std::vector<unsigned long long> off(blocks);
	unsigned long long total = 0;
	for (uint64_t b = 0; b < blocks; ++b) {
		off[b] = total;
		total += hc[b];
	}
	L->otfSet = true;
	L->otfFileEvents = nFileEvents;
	L->otfSelected = total;
	if (total > 0) {
		PWA_TRY(offsets.alloc(blocks * sizeof(unsigned long long), "OTF offsets"));
		PWA_TRY(L->otfIdx.alloc(total * sizeof(unsigned long long), "OTF indices"));
		PWA_TRY(cudaCheck(cudaMemcpyAsync(offsets.p, off.data(), blocks * sizeof(unsigned long long),
		                                  cudaMemcpyHostToDevice, s),
		                  "OTF offsets"));
		PWA_TRY(launchOtfCompact(a, offsets.as<unsigned long long>(), L->otfIdx.as<unsigned long long>(), s));
	}
	return cudaCheck(cudaStreamSynchronize(s), "OTF binning");
}

int pwa_likelihood_load_amp_files(pwa_likelihood* L, uint32_t nFiles, const char* const* paths, uint32_t nBinVars,
                                  const char* const* binVarNames, const double* lower, const double* upper)
{
	if (!L || !paths || nFiles == 0 || (nBinVars && (!binVarNames || !lower || !upper)))
		return setError(kErrArg, "null argument");
	if (!L->accAdded)
		return setError(kErrState, "no acceptance integral found; call addAccIntegral() before loading amplitudes");
	if (L->finished || L->nEvents != 0 || L->otfSet)
		return setError(kErrState, "amplitudes or a binning were already added");
	if (nBinVars > (uint32_t)kOtfMaxVars)
		return setError(kErrArg, "at most 8 binning variables");
	std::vector<AmpFile> files(nFiles);
	uint64_t total = 0;
	for (uint32_t f = 0; f < nFiles; ++f) {
		if (!paths[f])
			return setError(kErrArg, "null path");
		PWA_TRY(ampFileOpen(paths[f], files[f]));
		total += files[f].nEvents;
	}
	if (total == 0)
		return setError(kErrArg, "the amplitude files hold no events");
	auto find = [](const std::vector<std::string>& v, const std::string& name) -> int {
		for (size_t i = 0; i < v.size(); ++i)
			if (v[i] == name)
				return (int)i;
		return -1;
	};
	// every wave of the wave list must be in every file: finishInit refuses a
	// wave without amplitudes (pwaLikelihood.cc:1295-1302)
	std::vector<std::string> waves;
	for (const auto& kv : L->waveIdx)
		waves.push_back(kv.first);
	for (const auto& f : files)
		for (const auto& w : waves)
			if (find(f.waves, w) < 0)
				return setError(kErrArg, "could not find amplitude for wave '" + w + "' in file '" + f.path + "'");
	PWA_TRY(ensureDevice(L));
	cudaStream_t s = L->stream;
	if (nBinVars) {
		DevBuf vars;
		PWA_TRY(vars.alloc(nBinVars * total * sizeof(double), "binning variables"));
		std::vector<const double*> cols(nBinVars);
		for (uint32_t v = 0; v < nBinVars; ++v) {
			if (!binVarNames[v])
				return setError(kErrArg, "null binning variable name");
			uint64_t at = 0;
			for (const auto& f : files) {
				const int k = find(f.vars, binVarNames[v]);
				if (k < 0)
					return setError(kErrArg, std::string("binning variable '") + binVarNames[v] + "' is not in file '" +
					                             f.path + "'");
				PWA_TRY(ampFileToDevice(f, f.varOffset((uint32_t)k), f.nEvents * sizeof(double),
				                        vars.as<double>() + (size_t)v * total + at, s));
				at += f.nEvents;
			}
			cols[v] = vars.as<double>() + (size_t)v * total;
		}
		PWA_TRY(pwa_likelihood_set_otf_binning(L, nBinVars, lower, upper, cols.data(), total, PWA_MEMORY_DEVICE));
	}
	DevBuf row;
	PWA_TRY(row.alloc(total * sizeof(float2), "amplitude row"));
	for (const auto& w : waves) {
		uint64_t at = 0;
		for (const auto& f : files) {
			const int k = find(f.waves, w);
			PWA_TRY(ampFileToDevice(f, f.waveOffset((uint32_t)k), f.nEvents * sizeof(float2), row.as<float2>() + at, s));
			at += f.nEvents;
		}
		PWA_TRY(pwa_likelihood_add_amplitude(L, w.c_str(), row.p, total, PWA_COMPLEX64, PWA_MEMORY_DEVICE));
	}
	return kOk;
}

// Autotuner cache file: JSON with the device it was measured on and one
// object per tuned FdF shape, one per line:
//   {"device": "<name>", "fdf_plans": [
//   {"waves": W, "negative_waves": W0, "rank": R, "event_class": c, "stages": s, "variant": v},
//   ...]}
int pwa_autotune_cache_save(const char* path)
{
	if (!path)
		return setError(kErrArg, "null path");
	std::map<TuneKey, std::pair<int, int> > snap;
	{
		std::lock_guard<std::mutex> lock(g_tunedMutex);
		snap = g_tuned;
	}
	std::string dev = deviceName();
	for (char& c : dev)
		if (c == '"' || c == '\\')
			c = '_';
	FILE* fp = std::fopen(path, "w");
	if (!fp)
		return setError(kErrIo, std::string("cannot create '") + path + "'");
	std::fprintf(fp, "{\"device\": \"%s\", \"fdf_plans\": [\n", dev.c_str());
	size_t k = 0;
	for (const auto& kv : snap)
		std::fprintf(fp,
		             "{\"waves\": %u, \"negative_waves\": %u, \"rank\": %u, \"event_class\": %u, \"stages\": %d, "
		             "\"variant\": %d}%s\n",
		             kv.first.W, kv.first.W0, kv.first.R, kv.first.evClass, kv.second.first, kv.second.second,
		             ++k < snap.size() ? "," : "");
	std::fprintf(fp, "]}\n");
	if (std::fclose(fp) != 0)
		return setError(kErrIo, std::string("cannot write '") + path + "'");
	return kOk;
}

int pwa_autotune_cache_load(const char* path)
{
	if (!path)
		return setError(kErrArg, "null path");
	std::ifstream in(path);
	if (!in)
		return setError(kErrIo, std::string("cannot open '") + path + "'");
	std::string line;
	if (!std::getline(in, line))
		return setError(kErrIo, std::string("'") + path + "' is empty");
	const std::string tag = "{\"device\": \"";
	const size_t q = line.find('"', tag.size());
	if (line.compare(0, tag.size(), tag) != 0 || q == std::string::npos)
		return setError(kErrIo, std::string("'") + path + "' is not an autotuner cache");
	const std::string fileDev = line.substr(tag.size(), q - tag.size());
	std::string dev = deviceName();
	for (char& c : dev)
		if (c == '"' || c == '\\')
			c = '_';
	if (!dev.empty() && !fileDev.empty() && dev != fileDev)
		return setError(kErrArg, "autotuner cache '" + std::string(path) + "' was measured on " + fileDev +
		                             ", this device is " + dev);
	std::map<TuneKey, std::pair<int, int> > read;
	while (std::getline(in, line)) {
		if (line.compare(0, 2, "]}") == 0)
			break;
		unsigned W, W0, R, ev;
		int st, var;
		if (std::sscanf(line.c_str(),
		                "{\"waves\": %u, \"negative_waves\": %u, \"rank\": %u, \"event_class\": %u, \"stages\": %d, "
		                "\"variant\": %d}",
		                &W, &W0, &R, &ev, &st, &var) != 6 ||
		    st < 1 || st > 4 || var < 1 || var > 4 || W0 > W || R < 1)
			return setError(kErrIo, std::string("'") + path + "': malformed entry: " + line);
		read[TuneKey{W, W0, R, ev}] = std::make_pair(st, var);
	}
	std::lock_guard<std::mutex> lock(g_tunedMutex);
	for (const auto& kv : read)
		g_tuned[kv.first] = kv.second;
	return kOk;
}

int pwa_autotune_cache_clear(void)
{
	std::lock_guard<std::mutex> lock(g_tunedMutex);
	g_tuned.clear();
	return kOk;
}

int pwa_autotune_cache_size(uint32_t* n)
{
	if (!n)
		return setError(kErrArg, "null argument");
	std::lock_guard<std::mutex> lock(g_tunedMutex);
	*n = (uint32_t)g_tuned.size();
	return kOk;
}

int pwa_debug_fail_alloc_after(int64_t n)
{
	g_failAllocAfter.store(n < 0 ? -1 : (long)n);
	return kOk;
}

int pwa_likelihood_otf_selected(const pwa_likelihood* L, uint64_t* nSelected)
{
	if (!L || !nSelected)
		return setError(kErrArg, "null argument");
	*nSelected = L->otfSet ? L->otfSelected : 0;
	return kOk;
}

int pwa_likelihood_set_shard(pwa_likelihood* L, uint64_t totalEvents, int root)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	L->shardSet = true;
	L->shardTotal = totalEvents;
	L->shardRoot = root != 0;
	L->cacheValid = false;
	return kOk;
}

int pwa_likelihood_set_stream(pwa_likelihood* L, void* s)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	L->streamSet = true;
	if (L->ownStream && L->stream) {
		cudaStreamSynchronize(L->stream);
		cudaStreamDestroy(L->stream);
	}
	// NULL selects the CUDA default stream
	L->ownStream = false;
	L->stream = static_cast<cudaStream_t>(s);
	return kOk;
}

int pwa_likelihood_set_autotune(pwa_likelihood* L, int enable)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	L->autotune = enable != 0;
	return kOk;
}

int pwa_likelihood_plan(const pwa_likelihood* L, int* tileEvents, int* stages, int* blocks)
{
	PWA_TRY(checkFinished(L));
	if (tileEvents)
		*tileEvents = L->plan.E;
	if (stages)
		*stages = L->plan.stages;
	if (blocks)
		*blocks = L->plan.blocks;
	return kOk;
}

int pwa_likelihood_set_plan(pwa_likelihood* L, int stages)
{
	return pwa_likelihood_set_plan_variant(L, stages, 0);
}

int pwa_likelihood_set_plan_variant(pwa_likelihood* L, int stages, int phase1Events)
{
	PWA_TRY(checkFinished(L));
	if (phase1Events < 0 || phase1Events > 4)
		return setError(kErrArg,
		                "FdF kernel variant must be 1, 2 or 4 (events per lane), 3 (fused gradient) or 0 (keep)");
	const int ne = phase1Events ? phase1Events : L->plan.phase1Events;
	std::vector<FdfPlan> cands;
	PWA_TRY(planCandidates((int)L->nW[0], (int)L->W(), (int)L->rank, (int)L->storeB, L->nEvents, L->numSMs, L->maxSmem,
	                       &cands));
	for (const auto& c : cands)
		if (c.stages == stages && c.phase1Events == ne) {
			L->plan = c;
			return kOk;
		}
	return setError(kErrUnsupported, "no compiled FdF plan with this pipeline depth");
}

int pwa_likelihood_plan_variant(const pwa_likelihood* L, int* phase1Events)
{
	PWA_TRY(checkFinished(L));
	if (phase1Events)
		*phase1Events = L->plan.phase1Events;
	return kOk;
}

int pwa_likelihood_set_reduction(pwa_likelihood* L, int r)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (r != PWA_REDUCE_FP64 && r != PWA_REDUCE_KAHAN_FP32)
		return setError(kErrArg, "unknown reduction mode");
	L->reduction = r;
	return kOk;
}

// readWaveList + buildParDataStruct (pwaLikelihood.cc:1445-1556)
int pwa_likelihood_init(pwa_likelihood* L, uint32_t n, const char* const* names, const int32_t* refl,
                        const double* thresholds, uint32_t rank, double massBinCenter)
{
	if (!L || (!names && n) || (!refl && n))
		return setError(kErrArg, "null argument");
	if (L->initialized)
		return setError(kErrState, "likelihood already initialized");
	if (rank == 0)
		return setError(kErrArg, "rank must be at least 1");
	for (uint32_t i = 0; i < n; ++i) {
		if (refl[i] != 1 && refl[i] != -1)
			return setError(kErrArg, "reflectivity must be +1 or -1");
		const uint32_t e = refl[i] > 0 ? 1 : 0;
		if (L->waveIdx.count(names[i]))
			return setError(kErrArg, std::string("duplicate wave '") + names[i] + "'");
		L->waveIdx[names[i]] = std::make_pair(e, L->nW[e]);
		++L->nW[e];
		L->names[e].push_back(names[i]);
		L->thres[e].push_back(thresholds ? thresholds[i] : 0.);
	}
	if (L->nW[0] + L->nW[1] == 0)
		return setError(kErrArg, "no wave info");
	L->nWmax = std::max(L->nW[0], L->nW[1]);
	L->rank = rank;
	L->added[0].assign(L->nWmax, 0);
	L->added[1].assign(L->nWmax, 0);
	uint32_t P = 0;
	for (uint32_t r = 0; r < rank; ++r) {
		const int pos = (int)L->nW[1] - (int)r, neg = (int)L->nW[0] - (int)r;
		P += 2 * (std::max(pos - 1, 0) + std::max(neg - 1, 0));
		if (pos > 0)
			++P;
		if (neg > 0)
			++P;
	}
	P += 1;
	L->nPars = P;
	L->pars.assign(P, ParInfo());
	const uint32_t W = L->W();
	L->slotRe.assign((size_t)rank * W, -1);
	L->slotIm.assign((size_t)rank * W, -1);
	uint32_t p = 0;
	for (uint32_t r = 0; r < rank; ++r)
		for (uint32_t e = 0; e < 2; ++e)
			for (uint32_t w = 0; w < L->nW[e]; ++w) {
				const double th = L->thres[e][w];
				const bool fixed = (th != 0 && th >= massBinCenter);
				const size_t slot = (size_t)r * W + L->gw(e, w);
				if (w < r)
					continue;
				ParInfo pi;
				pi.waveName = L->names[e][w];
				pi.rank = (int)r;
				pi.threshold = th;
				pi.fixed = fixed;
				pi.realPart = true;
				L->pars[p] = pi;
				L->slotRe[slot] = (int)p;
				if (w == r) {
					p += 1;
				} else {
					pi.realPart = false;
					L->pars[p + 1] = pi;
					L->slotIm[slot] = (int)p + 1;
					p += 2;
				}
			}
	ParInfo flat;
	flat.waveName = "flat";
	L->pars[p] = flat;
	L->initialized = true;
	return kOk;
}

namespace {
// reorderIntegralMatrix (pwaLikelihood.cc:1562-1576): same-reflectivity blocks only
int reorder(const pwa_likelihood* L, const pwa_integral* I, std::vector<cplx>& out)
{
	out.assign((size_t)2 * L->nWmax * 2 * L->nWmax, cplx(0, 0));
	for (uint32_t e = 0; e < 2; ++e)
		for (uint32_t i = 0; i < L->nW[e]; ++i) {
			const int a = I->index(L->names[e][i]);
			if (a < 0)
				return setError(kErrArg, "cannot find wave '" + L->names[e][i] + "' in integral matrix");
			for (uint32_t j = 0; j < L->nW[e]; ++j) {
				const int b = I->index(L->names[e][j]);
				if (b < 0)
					return setError(kErrArg, "cannot find wave '" + L->names[e][j] + "' in integral matrix");
				out[L->mIdx(e, i, e, j)] = I->sums[(size_t)a * I->nWaves + b] / (double)I->nEvents;
			}
		}
	return kOk;
}
}  // namespace

int pwa_likelihood_add_norm_integral(pwa_likelihood* L, const pwa_integral* I)
{
	if (!L || !I)
		return setError(kErrArg, "null argument");
	if (!L->initialized)
		return setError(kErrState, "likelihood not initialized; call init() before addNormIntegral()");
	PWA_TRY(reorder(L, I, L->normM));
	L->numbAccEvents = I->nEvents;
	L->normAdded = true;
	return kOk;
}

int pwa_likelihood_add_acc_integral(pwa_likelihood* L, pwa_integral* I, uint64_t accEventsOverride)
{
	if (!L || !I)
		return setError(kErrArg, "null argument");
	if (!L->normAdded)
		return setError(kErrState,
		                "normalization integral not added before acceptance integral; call addNormIntegral() first");
	L->numbAccEvents = accEventsOverride == 0 ? L->numbAccEvents : accEventsOverride;
	L->totAcc = (double)I->nEvents / (double)L->numbAccEvents;
	I->nEvents = L->numbAccEvents;
	PWA_TRY(reorder(L, I, L->accM));
	L->accAdded = true;
	return kOk;
}

int pwa_likelihood_add_amplitude(pwa_likelihood* L, const char* waveName, const void* amps, uint64_t n, int ampType,
                                 int memory)
{
	if (!L || !waveName || !amps)
		return setError(kErrArg, "null argument");
	if (!L->accAdded)
		return setError(kErrState, "no acceptance integral found; call addAccIntegral() before addAmplitude()");
	if (ampType != PWA_COMPLEX64 && ampType != PWA_COMPLEX128)
		return setError(kErrArg, "unknown amplitude type");
	if (memory != PWA_MEMORY_HOST && memory != PWA_MEMORY_DEVICE)
		return setError(kErrArg, "unknown memory kind");
	if (L->finished)
		return setError(kErrState, "finishInit() already called");
	auto it = L->waveIdx.find(waveName);
	if (it == L->waveIdx.end())
		return setError(kErrArg, std::string("requested to add decay amplitudes for wave '") + waveName +
		                             "' which is not in wavelist");
	if (n == 0)
		return setError(kErrArg, "no events to load");
	PWA_TRY(ensureDevice(L));
	cudaStream_t s = L->stream;
	// on-the-fly binning: keep the selected events of the file, in order
	DevBuf otfFull, otfSel;
	if (L->otfSet) {
		if (n != L->otfFileEvents)
			return setError(kErrArg, "amplitude array length differs from the event count of the on-the-fly binning");
		if (L->otfSelected == 0)
			return setError(kErrArg, "no event of the data file is in the on-the-fly bin");
		const int elem = (ampType == PWA_COMPLEX128) ? 16 : 8;
		const void* src = amps;
		if (memory == PWA_MEMORY_HOST) {
			PWA_TRY(otfFull.alloc(n * elem, "amplitude upload"));
			PWA_TRY(cudaCheck(cudaMemcpyAsync(otfFull.p, amps, n * elem, cudaMemcpyHostToDevice, s), "upload"));
			src = otfFull.p;
		} else {
			PWA_TRY(cudaCheck(cudaDeviceSynchronize(), "synchronise before reading device amplitudes"));
		}
		PWA_TRY(otfSel.alloc(L->otfSelected * elem, "selected amplitudes"));
		PWA_TRY(launchOtfGather(src, L->otfIdx.as<unsigned long long>(), L->otfSelected, elem, otfSel.p, s));
		PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "OTF gather"));
		amps = otfSel.p;
		memory = PWA_MEMORY_DEVICE;
		n = L->otfSelected;
	}
	if (L->nEvents == 0) {
		L->nEvents = n;
		L->storeB = (uint32_t)chooseStoreBlock((int)L->W(), (int)L->rank, L->maxSmem);
		const uint64_t nBlocks = (n + L->storeB - 1) / L->storeB;
		PWA_TRY(L->amps.alloc((size_t)nBlocks * L->W() * L->storeB * sizeof(float2), "amplitude store"));
		PWA_TRY(cudaCheck(cudaMemsetAsync(L->amps.p, 0, L->amps.bytes, s), "amplitude store memset"));
		PWA_TRY(L->dFlag.alloc(sizeof(unsigned), "flag"));
	}
	if (n != L->nEvents)
		return setError(kErrArg, "size mismatch in amplitude arrays");
	const uint32_t e = it->second.first, w = it->second.second;
	const cplx normInt = L->normM[L->mIdx(e, w, e, w)];
	bool fixPar = (L->accM[L->mIdx(e, w, e, w)] == 0.);
	const double divisor = (L->useNormalizedAmps && normInt != 0.) ? std::sqrt(normInt.real()) : 1.;
	const uint32_t gwave = L->gw(e, w);
	bool anyNonZero = false;
	if (memory == PWA_MEMORY_HOST) {
		// convert in FP64 on the host, upload through a pinned staging buffer
		// into a contiguous device row, then scatter it into the tiled store
		const size_t chunk = 1 << 20;
		PinnedBuf stage;
		PWA_TRY(stage.ensure(chunk * sizeof(float2), "staging"));
		PWA_TRY(L->ampTmp.ensure(n * sizeof(float2), "amplitude row"));
		float2* row = L->ampTmp.as<float2>();
		for (uint64_t b = 0; b < n; b += chunk) {
			const uint64_t m = std::min<uint64_t>(chunk, n - b);
			float2* dst = stage.as<float2>();
			for (uint64_t i = 0; i < m; ++i) {
				double re, im;
				if (ampType == PWA_COMPLEX128) {
					re = static_cast<const double*>(amps)[2 * (b + i)];
					im = static_cast<const double*>(amps)[2 * (b + i) + 1];
				} else {
					re = static_cast<const float*>(amps)[2 * (b + i)];
					im = static_cast<const float*>(amps)[2 * (b + i) + 1];
				}
				anyNonZero = anyNonZero || re != 0. || im != 0.;
				dst[i] = make_float2((float)(re / divisor), (float)(im / divisor));
			}
			PWA_TRY(cudaCheck(cudaMemcpyAsync(row + b, dst, m * sizeof(float2), cudaMemcpyHostToDevice, s),
			                  "amplitude upload"));
			PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "amplitude upload sync"));
		}
		PWA_TRY(launchConvertRow(row, 0, L->amps.as<float2>(), L->W(), gwave, L->storeB, n, 1.0, L->dFlag.as<unsigned>(),
		                         s));
		PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "amplitude scatter sync"));
	} else {
		// the caller's streams may still be writing the device amplitudes
		PWA_TRY(cudaCheck(cudaDeviceSynchronize(), "synchronise before reading device amplitudes"));
		PWA_TRY(cudaCheck(cudaMemsetAsync(L->dFlag.p, 0, sizeof(unsigned), s), "memset"));
		PWA_TRY(launchConvertRow(amps, ampType == PWA_COMPLEX128 ? 1 : 0, L->amps.as<float2>(), L->W(), gwave, L->storeB, n,
		                         divisor, L->dFlag.as<unsigned>(), s));
		unsigned flag = 0;
		PWA_TRY(cudaCheck(cudaMemcpyAsync(&flag, L->dFlag.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "flag"));
		PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "amplitude convert sync"));
		anyNonZero = flag != 0;
	}
	if (L->useNormalizedAmps && normInt == 0. && anyNonZero)
		return setError(kErrArg, std::string("normalization integral for wave '") + waveName +
		                             "' is zero, but the amplitude is not");
	if (anyNonZero)
		fixPar = false;
	if (fixPar)
		for (auto& p : L->pars)
			if (p.waveName == waveName)
				p.fixed = true;
	L->added[e][w] = 1;
	return kOk;
}

int pwa_likelihood_finish_init(pwa_likelihood* L)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (!L->accAdded)
		return setError(kErrState, "integrals not added");
	for (uint32_t e = 0; e < 2; ++e)
		for (uint32_t w = 0; w < L->nW[e]; ++w)
			if (!L->added[e][w])
				return setError(kErrState, "not all expected amplitudes were added to the likelihood ('" +
				                               L->names[e][w] + "')");
	// phase-space integrals and rescaling (pwaLikelihood.cc:1303-1335)
	L->psInt.assign((size_t)2 * L->nWmax, 0.);
	for (uint32_t e = 0; e < 2; ++e)
		for (uint32_t w = 0; w < L->nW[e]; ++w)
			L->psInt[e * L->nWmax + w] = std::sqrt(L->normM[L->mIdx(e, w, e, w)].real());
	if (L->useNormalizedAmps) {
		for (uint32_t e1 = 0; e1 < 2; ++e1)
			for (uint32_t i = 0; i < L->nW[e1]; ++i) {
				double ni = std::sqrt(L->normM[L->mIdx(e1, i, e1, i)].real());
				if (ni == 0)
					ni = 1;
				for (uint32_t e2 = 0; e2 < 2; ++e2)
					for (uint32_t j = 0; j < L->nW[e2]; ++j) {
						double nj = std::sqrt(L->normM[L->mIdx(e2, j, e2, j)].real());
						if (nj == 0)
							nj = 1;
						if (e1 != e2 || i != j)
							L->normM[L->mIdx(e1, i, e2, j)] /= ni * nj;
						L->accM[L->mIdx(e1, i, e2, j)] /= ni * nj;
					}
			}
		for (uint32_t e = 0; e < 2; ++e)
			for (uint32_t w = 0; w < L->nW[e]; ++w)
				if (L->normM[L->mIdx(e, w, e, w)] != 0.)
					L->normM[L->mIdx(e, w, e, w)] = 1.;
	}
	// device-side evaluation resources
	PWA_TRY(ensureDevice(L));
	const uint32_t W = L->W();
	std::vector<FdfPlan> cands;
	PWA_TRY(planCandidates((int)L->nW[0], (int)W, (int)L->rank, (int)L->storeB, L->nEvents, L->numSMs, L->maxSmem,
	                       &cands));
	L->plan = cands.front();
	L->ampTmp.release();
	const size_t nSlot = (size_t)L->rank * W;
	const size_t nPartial = 2 + 2 * nSlot;
	PWA_TRY(L->dSlotRe.alloc(nSlot * sizeof(int), "slot map"));
	PWA_TRY(L->dSlotIm.alloc(nSlot * sizeof(int), "slot map"));
	PWA_TRY(L->dFixAcc.alloc(fdfAccumulatorWords((int)nPartial) * sizeof(unsigned long long), "fixed-point accumulators"));
	PWA_TRY(L->dNfAcc.alloc(nPartial * sizeof(double), "non-finite accumulators"));
	PWA_TRY(L->dCounter.alloc(sizeof(unsigned), "arrival counter"));
	PWA_TRY(L->dErr.alloc(sizeof(unsigned), "error flag"));
	PWA_TRY(L->dPar.alloc(L->nPars * sizeof(double), "parameters"));
	PWA_TRY(L->dOut.alloc((L->nPars + 2) * sizeof(double), "result"));
	// mapped: the host-buffer entry points let the kernel read the
	// parameters from and write the results to host memory directly
	PWA_TRY(L->hPar.ensure(L->nPars * sizeof(double), "pinned parameters", true));
	PWA_TRY(L->hOut.ensure((L->nPars + 2) * sizeof(double), "pinned result", true));
	std::vector<double> accI;
	for (uint32_t e = 0; e < 2; ++e)
		for (uint32_t i = 0; i < L->nW[e]; ++i)
			for (uint32_t j = 0; j < L->nW[e]; ++j) {
				const cplx v = L->accM[L->mIdx(e, i, e, j)];
				accI.push_back(v.real());
				accI.push_back(v.imag());
			}
	PWA_TRY(L->dAccI.alloc(std::max<size_t>(accI.size(), 2) * sizeof(double), "acceptance integral"));
	cudaStream_t s = L->stream;
	if (!accI.empty())
		PWA_TRY(cudaCheck(cudaMemcpyAsync(L->dAccI.p, accI.data(), accI.size() * sizeof(double),
		                                  cudaMemcpyHostToDevice, s),
		                  "acc upload"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(L->dSlotRe.p, L->slotRe.data(), nSlot * sizeof(int), cudaMemcpyHostToDevice, s),
	                  "slot upload"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(L->dSlotIm.p, L->slotIm.data(), nSlot * sizeof(int), cudaMemcpyHostToDevice, s),
	                  "slot upload"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(L->dCounter.p, 0, L->dCounter.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(L->dFixAcc.p, 0, L->dFixAcc.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(L->dNfAcc.p, 0, L->dNfAcc.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(L->dErr.p, 0, sizeof(unsigned), s), "memset"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "finishInit sync"));
	if (L->autotune && cands.size() > 1 && L->nEvents >= 65536)
		PWA_TRY(autotunePlan(L, cands));
	L->finished = true;
	return kOk;
}

int pwa_likelihood_nmb_pars(const pwa_likelihood* L, uint32_t* n)
{
	if (!L || !n)
		return setError(kErrArg, "null argument");
	*n = L->nPars;
	return kOk;
}

int pwa_likelihood_nmb_pars_fixed(const pwa_likelihood* L, uint32_t* n)
{
	if (!L || !n)
		return setError(kErrArg, "null argument");
	uint32_t k = 0;
	for (const auto& p : L->pars)
		k += p.fixed ? 1 : 0;
	*n = k;
	return kOk;
}

int pwa_likelihood_nmb_events(const pwa_likelihood* L, uint64_t* n)
{
	if (!L || !n)
		return setError(kErrArg, "null argument");
	*n = L->nEvents;
	return kOk;
}

int pwa_likelihood_rank(const pwa_likelihood* L, uint32_t* r)
{
	if (!L || !r)
		return setError(kErrArg, "null argument");
	*r = L->rank;
	return kOk;
}

int pwa_likelihood_nmb_waves(const pwa_likelihood* L, int refl, uint32_t* n)
{
	if (!L || !n)
		return setError(kErrArg, "null argument");
	*n = (refl == 0) ? L->W() : (refl > 0 ? L->nW[1] : L->nW[0]);
	return kOk;
}

int pwa_likelihood_parameter(const pwa_likelihood* L, uint32_t i, char* nameBuf, uint32_t bufLen, int* fixed,
                             int* realPart, int32_t* rank, double* threshold)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (i >= L->nPars)
		return setError(kErrArg, "parameter index out of range");
	const ParInfo& p = L->pars[i];
	if (nameBuf && bufLen) {
		// fitParameter::parName (pwaLikelihood.cc:107-122)
		std::ostringstream o;
		o << "V";
		if (p.waveName != "flat")
			o << p.rank;
		o << "_" << p.waveName << (p.realPart ? "_RE" : "_IM");
		std::snprintf(nameBuf, bufLen, "%s", o.str().c_str());
	}
	if (fixed)
		*fixed = p.fixed ? 1 : 0;
	if (realPart)
		*realPart = p.realPart ? 1 : 0;
	if (rank)
		*rank = p.rank;
	if (threshold)
		*threshold = p.threshold;
	return kOk;
}

int pwa_likelihood_tot_acc(const pwa_likelihood* L, double* t)
{
	if (!L || !t)
		return setError(kErrArg, "null argument");
	*t = L->totAcc;
	return kOk;
}

int pwa_likelihood_fdf(pwa_likelihood* L, const double* par, double* f, double* grad)
{
	if (!par || !f || !grad)
		return setError(kErrArg, "null argument");
	return hostEval(L, par, f, grad, 1, PWA_CALL_FDF);
}

int pwa_likelihood_doeval(pwa_likelihood* L, const double* par, double* f)
{
	if (!par || !f)
		return setError(kErrArg, "null argument");
	return hostEval(L, par, f, nullptr, 0, PWA_CALL_DOEVAL);
}

int pwa_likelihood_gradient(pwa_likelihood* L, const double* par, double* grad)
{
	if (!par || !grad)
		return setError(kErrArg, "null argument");
	return hostEval(L, par, nullptr, grad, 1, PWA_CALL_GRADIENT);
}

int pwa_likelihood_doderivative(pwa_likelihood* L, const double* par, uint32_t index, double* d)
{
	PWA_TRY(checkFinished(L));
	if (!par || !d)
		return setError(kErrArg, "null argument");
	if (index >= L->nPars)
		return setError(kErrArg, "derivative index out of range");
	++L->info[PWA_CALL_DODERIVATIVE].nCalls;
	if (L->cacheValid && std::equal(par, par + L->nPars, L->parCache.begin())) {
		*d = L->derivCache[index];
		return kOk;
	}
	std::vector<double> g(L->nPars);
	double f;
	PWA_TRY(hostEval(L, par, &f, g.data(), 1, PWA_CALL_FDF));
	*d = g[index];
	return kOk;
}

int pwa_likelihood_fdf_batch(pwa_likelihood* L, uint32_t nPoints, const double* par, double* f, double* grad)
{
	PWA_TRY(checkFinished(L));
	if (!par || !f || !grad)
		return setError(kErrArg, "null argument");
	if (nPoints == 0)
		return kOk;
	const uint32_t P = L->nPars;
	const double t0 = seconds();
	PWA_TRY(L->dPar.ensure((size_t)nPoints * P * sizeof(double), "batch parameters"));
	PWA_TRY(L->dOut.ensure((size_t)nPoints * (P + 2) * sizeof(double), "batch results"));
	PWA_TRY(L->hPar.ensure((size_t)nPoints * P * sizeof(double), "pinned batch parameters", true));
	PWA_TRY(L->hOut.ensure((size_t)nPoints * (P + 2) * sizeof(double), "pinned batch results", true));
	std::memcpy(L->hPar.p, par, (size_t)nPoints * P * sizeof(double));
	cudaStream_t s = L->stream;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(L->dPar.p, L->hPar.p, (size_t)nPoints * P * sizeof(double),
	                                  cudaMemcpyHostToDevice, s),
	                  "H2D batch"));
	for (uint32_t k = 0; k < nPoints; ++k)
		PWA_TRY(launchEval(L, L->dPar.as<double>() + (size_t)k * P, L->dOut.as<double>() + (size_t)k * (P + 2), 1, s));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(L->hOut.p, L->dOut.p, (size_t)nPoints * (P + 2) * sizeof(double),
	                                  cudaMemcpyDeviceToHost, s),
	                  "D2H batch"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "batch sync"));
	const double* out = L->hOut.as<double>();
	for (uint32_t k = 0; k < nPoints; ++k) {
		if (out[(size_t)k * (P + 2) + P + 1] != 0.) {
			cudaMemsetAsync(L->dErr.p, 0, sizeof(unsigned), s);
			cudaStreamSynchronize(s);
			return setError(kErrTimeout, "a bounded device-side wait expired in the FdF kernel");
		}
		f[k] = out[(size_t)k * (P + 2)];
		std::memcpy(grad + (size_t)k * P, out + (size_t)k * (P + 2) + 1, P * sizeof(double));
	}
	CallInfo& ci = L->info[PWA_CALL_FDF];
	ci.nCalls += nPoints;
	ci.total += seconds() - t0;
	return kOk;
}

int pwa_likelihood_fdf_device(pwa_likelihood* L, const double* dPar, double* dOut, int withGradient, void* stream)
{
	PWA_TRY(checkFinished(L));
	if (!dPar || !dOut)
		return setError(kErrArg, "null argument");
	cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : L->stream;
	return launchEval(L, dPar, dOut, withGradient ? 1 : 0, s);
}

int pwa_likelihood_hessian(pwa_likelihood* L, const double* par, double* H)
{
	PWA_TRY(checkFinished(L));
	if (!par || !H)
		return setError(kErrArg, "null argument");
	const double t0 = seconds();
	const uint32_t P = L->nPars, W = L->W(), R = L->rank;
	const uint32_t nS = R * W, nY1 = 2 * nS + 1, nY2 = W + 1;
	cudaStream_t s = L->stream;
	// event slabs sized so that the [d; conj d; 1] columns stay below ~1 GB
	uint64_t slab = (uint64_t)1 << 30;
	slab /= (uint64_t)nY1 * sizeof(float2);
	slab = std::max<uint64_t>(1024, std::min<uint64_t>(slab, (L->nEvents + 63) / 64 * 64));
	const int tps = ((int)nY1 + 63) / 64;
	const int nTiles = tps * (tps + 1) / 2;
	int chunks = std::max(1, (4 * L->numSMs + nTiles - 1) / nTiles);
	chunks = (int)std::min<uint64_t>((uint64_t)chunks, std::max<uint64_t>(1, slab / 64));
	DevBuf dY1, dY2, dW1, dW2, dPart, dG1, dG2, dHP;
	PWA_TRY(dY1.alloc((size_t)nY1 * slab * sizeof(float2), "hessian operand"));
	PWA_TRY(dY2.alloc((size_t)nY2 * slab * sizeof(float2), "hessian operand"));
	PWA_TRY(dW1.alloc(slab * sizeof(double), "hessian weights"));
	PWA_TRY(dW2.alloc(slab * sizeof(double), "hessian weights"));
	PWA_TRY(dPart.alloc((size_t)chunks * nY1 * nY1 * 2 * sizeof(double), "hessian partials"));
	PWA_TRY(dG1.alloc((size_t)nY1 * nY1 * 2 * sizeof(double), "hessian gram"));
	PWA_TRY(dG2.alloc((size_t)nY2 * nY2 * 2 * sizeof(double), "hessian gram"));
	PWA_TRY(dHP.alloc(P * sizeof(double), "hessian parameters"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(dHP.p, par, P * sizeof(double), cudaMemcpyHostToDevice, s), "H2D par"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dG1.p, 0, dG1.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dG2.p, 0, dG2.bytes, s), "memset"));
	for (uint64_t e0 = 0; e0 < L->nEvents; e0 += slab) {
		const uint64_t K = std::min<uint64_t>(slab, L->nEvents - e0);
		PWA_TRY(launchHessPrep(L->amps.as<float2>(), L->nEvents, L->storeB, e0, slab, (int)L->nW[0], (int)W, (int)R,
		                       (int)P, dHP.as<double>(), L->dSlotRe.as<int>(), L->dSlotIm.as<int>(), dY1.as<float2>(),
		                       dY2.as<float2>(), dW1.as<double>(), dW2.as<double>(), s));
		const int ck = (int)std::min<uint64_t>((uint64_t)chunks, std::max<uint64_t>(1, K / 64));
		GramArgs g{};
		g.K = K;
		g.ldK = slab;
		g.partials = dPart.as<double>();
		g.chunks = ck;
		g.amps = dY1.as<float2>();
		g.W = (int)nY1;
		g.weightK = dW1.as<double>();
		PWA_TRY(launchGramSimt(g, PWA_PRECISION_FP32, s));
		PWA_TRY(launchGramReduce(g.partials, ck, (int)nY1, dG1.as<double>(), 1, s));
		g.amps = dY2.as<float2>();
		g.W = (int)nY2;
		g.weightK = dW2.as<double>();
		PWA_TRY(launchGramSimt(g, PWA_PRECISION_FP32, s));
		PWA_TRY(launchGramReduce(g.partials, ck, (int)nY2, dG2.as<double>(), 1, s));
	}
	std::vector<double> G1((size_t)nY1 * nY1 * 2), G2((size_t)nY2 * nY2 * 2);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(G1.data(), dG1.p, G1.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(G2.data(), dG2.p, G2.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "hessian sync"));
	auto g1 = [&](uint32_t a, uint32_t b) { return cplx(G1[((size_t)a * nY1 + b) * 2], G1[((size_t)a * nY1 + b) * 2 + 1]); };
	auto g2 = [&](uint32_t a, uint32_t b) { return cplx(G2[((size_t)a * nY2 + b) * 2], G2[((size_t)a * nY2 + b) * 2 + 1]); };

	// assemble the reference's [slot][slot][3] blocks (pwaLikelihood.cc:736-800)
	std::vector<cplx> V;
	double flat;
	fromPar(L, par, V, flat);
	const double nEvt = normFactor(L);
	const double twice = 2. * nEvt;
	std::vector<double> h((size_t)nS * nS * 3);
	for (uint32_t si = 0; si < nS; ++si) {
		const uint32_t ri = si / W, gi = si % W, ei = gi < L->nW[0] ? 0 : 1;
		for (uint32_t sj = 0; sj < nS; ++sj) {
			const uint32_t rj = sj / W, gj = sj % W, ej = gj < L->nW[0] ? 0 : 1;
			const cplx Gd = g1(si, sj), Gn = g1(si, nS + sj);
			double h0 = 0.5 * (Gd.real() + Gn.real());
			double h1 = 0.5 * (Gn.imag() - Gd.imag());
			double h2 = 0.5 * (Gd.real() - Gn.real());
			if (ri == rj && ei == ej) {
				const cplx M = g2(gi, gj);
				const uint32_t li = gi - (ei ? L->nW[0] : 0), lj = gj - (ej ? L->nW[0] : 0);
				const cplx I = L->accM[L->mIdx(ei, li, ei, lj)];
				h0 += -M.real() + I.real() * twice;
				h1 += -M.imag() + I.imag() * twice;
				h2 += -M.real() + I.real() * twice;
			}
			double* hh = &h[((size_t)si * nS + sj) * 3];
			hh[0] = h0;
			hh[1] = h1;
			hh[2] = h2;
		}
	}
	std::vector<cplx> flatTerms(nS);
	for (uint32_t si = 0; si < nS; ++si)
		flatTerms[si] = flat * g1(si, 2 * nS);
	double hFlat = flat * flat * g1(2 * nS, 2 * nS).real() - g2(W, W).real() + twice * L->totAcc;
	if (priorOf(L) == PWA_PRIOR_HALF_CAUCHY) {
		// pwaLikelihood.cc:766-798
		const double gw = L->cauchyWidth, g2w = gw * gw;
		for (uint32_t si = 0; si < nS; ++si) {
			const cplx v = V[si];
			const double rr = std::abs(v);
			const double cf = 1. / (1. + (rr * rr) / g2w);
			const double cd = (-2. * rr * g2w) / ((g2w + rr * rr) * (g2w + rr * rr));
			const double cd2 = g2w / ((g2w + rr * rr) * (g2w + rr * rr)) * (-2. + 8. * rr * rr / (g2w + rr * rr));
			const double a1 = cd2 / (cf * rr * rr);
			const double a2 = cd * cd / (cf * cf * rr * rr);
			const double a3 = cd / (cf * rr);
			const double a4 = cd / (cf * rr * rr * rr);
			const double a124 = a1 - a2 - a4;
			double* hh = &h[((size_t)si * nS + si) * 3];
			hh[0] -= a124 * v.real() * v.real() + a3;
			hh[1] -= a124 * v.real() * v.imag();
			hh[2] -= a124 * v.imag() * v.imag() + a3;
		}
	}
	// map onto the parameter layout (pwaLikelihood.cc:802-850)
	std::fill(H, H + (size_t)P * P, 0.);
	for (uint32_t si = 0; si < nS; ++si) {
		const int r1 = L->slotRe[si], i1 = L->slotIm[si];
		if (r1 < 0 || L->pars[r1].fixed)
			continue;
		for (uint32_t sj = 0; sj < nS; ++sj) {
			const int r2 = L->slotRe[sj], i2 = L->slotIm[sj];
			if (r2 < 0 || L->pars[r2].fixed)
				continue;
			H[(size_t)r1 * P + r2] = h[((size_t)si * nS + sj) * 3 + 0];
			if (i2 >= 0)
				H[(size_t)r1 * P + i2] = h[((size_t)si * nS + sj) * 3 + 1];
			if (i1 >= 0)
				H[(size_t)i1 * P + r2] = h[((size_t)sj * nS + si) * 3 + 1];
			if (i1 >= 0 && i2 >= 0)
				H[(size_t)i1 * P + i2] = h[((size_t)si * nS + sj) * 3 + 2];
		}
		H[(size_t)r1 * P + P - 1] = flatTerms[si].real();
		H[(size_t)(P - 1) * P + r1] = flatTerms[si].real();
		if (i1 >= 0) {
			H[(size_t)i1 * P + P - 1] = flatTerms[si].imag();
			H[(size_t)(P - 1) * P + i1] = flatTerms[si].imag();
		}
	}
	H[(size_t)(P - 1) * P + P - 1] = hFlat;
	CallInfo& ci = L->info[PWA_CALL_HESSIAN];
	++ci.nCalls;
	ci.total += seconds() - t0;
	return kOk;
}

int pwa_likelihood_covariance_matrix(const pwa_likelihood* L, const double* H, double* C)
{
	PWA_TRY(checkFinished(L));
	if (!H || !C)
		return setError(kErrArg, "null argument");
	// invert the free-parameter block (pwaLikelihood.cc:929-981); Gauss-Jordan
	// with partial pivoting in FP64 on the host (P x P, once per fit)
	const uint32_t P = L->nPars;
	std::vector<uint32_t> fr;
	for (uint32_t i = 0; i < P; ++i)
		if (!L->pars[i].fixed)
			fr.push_back(i);
	const size_t n = fr.size();
	std::vector<double> a(n * n), inv(n * n, 0.);
	for (size_t i = 0; i < n; ++i) {
		for (size_t j = 0; j < n; ++j)
			a[i * n + j] = H[(size_t)fr[i] * P + fr[j]];
		inv[i * n + i] = 1.;
	}
	for (size_t c = 0; c < n; ++c) {
		size_t piv = c;
		for (size_t r = c + 1; r < n; ++r)
			if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c]))
				piv = r;
		if (a[piv * n + c] == 0.)
			return setError(kErrNumerical, "Hessian is singular");
		if (piv != c)
			for (size_t k = 0; k < n; ++k) {
				std::swap(a[c * n + k], a[piv * n + k]);
				std::swap(inv[c * n + k], inv[piv * n + k]);
			}
		const double d = a[c * n + c];
		for (size_t k = 0; k < n; ++k) {
			a[c * n + k] /= d;
			inv[c * n + k] /= d;
		}
		for (size_t r = 0; r < n; ++r) {
			if (r == c)
				continue;
			const double fct = a[r * n + c];
			if (fct == 0.)
				continue;
			for (size_t k = 0; k < n; ++k) {
				a[r * n + k] -= fct * a[c * n + k];
				inv[r * n + k] -= fct * inv[c * n + k];
			}
		}
	}
	std::fill(C, C + (size_t)P * P, 0.);
	for (size_t i = 0; i < n; ++i)
		for (size_t j = 0; j < n; ++j)
			C[(size_t)fr[i] * P + fr[j]] = inv[i * n + j];
	return kOk;
}

int pwa_likelihood_correct_param_signs(const pwa_likelihood* L, const double* par, double* out)
{
	if (!L || !par || !out)
		return setError(kErrArg, "null argument");
	if (!L->initialized)
		return setError(kErrState, "likelihood not initialized");
	// pwaLikelihood.cc:986-1010
	std::vector<cplx> V;
	double flat;
	fromPar(L, par, V, flat);
	if (flat < 0)
		flat *= -1;
	const uint32_t W = L->W();
	for (uint32_t r = 0; r < L->rank; ++r)
		for (uint32_t e = 0; e < 2; ++e) {
			if (r >= L->nW[e])
				continue;  // anchor wave absent in this reflectivity: V == 0, nothing to flip
			const cplx anchor = V[(size_t)r * W + L->gw(e, r)];
			if (anchor.real() < 0 && anchor.imag() == 0)
				for (uint32_t w = 0; w < L->nW[e]; ++w)
					V[(size_t)r * W + L->gw(e, w)] *= -1;
		}
	toPar(L, V, flat, out);
	return kOk;
}

int pwa_likelihood_integral_matrices(const pwa_likelihood* L, double* norm, double* acc, double* ps, int withFlat)
{
	PWA_TRY(checkFinished(L));
	if (!norm || !acc || !ps)
		return setError(kErrArg, "null argument");
	const uint32_t n = L->W(), sz = n + (withFlat ? 1 : 0);
	std::fill(norm, norm + 2 * (size_t)sz * sz, 0.);
	std::fill(acc, acc + 2 * (size_t)sz * sz, 0.);
	std::fill(ps, ps + sz, 0.);
	uint32_t ii = 0;
	for (uint32_t e1 = 0; e1 < 2; ++e1)
		for (uint32_t i = 0; i < L->nW[e1]; ++i, ++ii) {
			ps[ii] = L->psInt[e1 * L->nWmax + i];
			uint32_t jj = 0;
			for (uint32_t e2 = 0; e2 < 2; ++e2)
				for (uint32_t j = 0; j < L->nW[e2]; ++j, ++jj) {
					const cplx nv = L->normM[L->mIdx(e1, i, e2, j)], av = L->accM[L->mIdx(e1, i, e2, j)];
					norm[2 * ((size_t)ii * sz + jj)] = nv.real();
					norm[2 * ((size_t)ii * sz + jj) + 1] = nv.imag();
					acc[2 * ((size_t)ii * sz + jj)] = av.real();
					acc[2 * ((size_t)ii * sz + jj) + 1] = av.imag();
				}
		}
	if (withFlat) {
		norm[2 * ((size_t)n * sz + n)] = 1.;
		acc[2 * ((size_t)n * sz + n)] = L->totAcc;
		ps[n] = 1.;
	}
	return kOk;
}

int pwa_likelihood_build_prod_amp_arrays(const pwa_likelihood* L, const double* par, double* prodAmps,
                                         int32_t* parIndices, uint32_t* nAmps, int withFlat)
{
	if (!L || !par || !prodAmps || !parIndices || !nAmps)
		return setError(kErrArg, "null argument");
	if (!L->initialized)
		return setError(kErrState, "likelihood not initialized");
	// pwaLikelihood.cc:1626-1665
	uint32_t p = 0, k = 0;
	for (uint32_t r = 0; r < L->rank; ++r)
		for (uint32_t e = 0; e < 2; ++e)
			for (uint32_t w = 0; w < L->nW[e]; ++w) {
				if (w < r)
					continue;
				double re, im;
				if (w == r) {
					parIndices[2 * k] = (int32_t)p;
					parIndices[2 * k + 1] = -1;
					re = par[p];
					im = 0;
					p += 1;
				} else {
					parIndices[2 * k] = (int32_t)p;
					parIndices[2 * k + 1] = (int32_t)p + 1;
					re = par[p];
					im = par[p + 1];
					p += 2;
				}
				prodAmps[2 * k] = re;
				prodAmps[2 * k + 1] = im;
				++k;
			}
	if (withFlat) {
		prodAmps[2 * k] = par[p];
		prodAmps[2 * k + 1] = 0.;
		parIndices[2 * k] = (int32_t)p;
		parIndices[2 * k + 1] = -1;
		++k;
	}
	*nAmps = k;
	return kOk;
}

int pwa_likelihood_func_call_info(const pwa_likelihood* L, int call, uint64_t* nCalls, double* total, double* func,
                                  double* norm)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (call < 0 || call > PWA_CALL_HESSIAN)
		return setError(kErrArg, "unknown call type");
	const CallInfo& c = L->info[call];
	if (nCalls)
		*nCalls = c.nCalls;
	if (total)
		*total = c.total;
	if (func)
		*func = c.func;
	if (norm)
		*norm = c.norm;
	return kOk;
}

int pwa_likelihood_set_timing(pwa_likelihood* L, int enable)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (enable && L->timingEvents.empty()) {
		PWA_TRY(ensureDevice(L));
		const size_t n = 2 * 65536;
		L->timingEvents.resize(n, nullptr);
		for (auto& e : L->timingEvents)
			PWA_TRY(cudaCheck(cudaEventCreate(&e), "timing event create"));
	}
	L->timing = enable != 0;
	L->nTimed = 0;
	return kOk;
}

int pwa_likelihood_kernel_times(pwa_likelihood* L, double* mainMs, double* finMs, uint64_t* nTimed)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	double a = 0., b = 0.;
	if (L->nTimed > 0)
		PWA_TRY(cudaCheck(cudaEventSynchronize(L->timingEvents[2 * L->nTimed - 1]), "timing sync"));
	for (size_t k = 0; k < L->nTimed; ++k) {
		float x = 0.f;
		PWA_TRY(cudaCheck(cudaEventElapsedTime(&x, L->timingEvents[2 * k], L->timingEvents[2 * k + 1]), "elapsed"));
		a += x;
	}
	if (mainMs)
		*mainMs = a;
	if (finMs)
		*finMs = b;
	if (nTimed)
		*nTimed = L->nTimed;
	L->nTimed = 0;
	return kOk;
}

int pwa_likelihood_reset_func_call_info(pwa_likelihood* L)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	for (auto& c : L->info)
		c = CallInfo();
	return kOk;
}

}  // extern "C"

// ===========================================================================
// Read-only device view of a finished likelihood
// ===========================================================================
namespace pwa {

int likelihoodView(const pwa_likelihood* L, LikelihoodView* v)
{
	PWA_TRY(checkFinished(L));
	v->amps = L->amps.as<float2>();
	v->nEvents = L->nEvents;
	v->storeB = L->storeB;
	v->W0 = (int)L->nW[0];
	v->W = (int)L->W();
	v->R = (int)L->rank;
	v->P = (int)L->nPars;
	v->slotRe = L->slotRe;
	v->slotIm = L->slotIm;
	v->accI = L->dAccI.as<double>();
	v->nEvt = normFactor(L);
	v->totAcc = L->totAcc;
	v->prior = priorOf(L);
	v->cauchyWidth = L->cauchyWidth;
	v->device = L->device;
	return kOk;
}

}  // namespace pwa

// ===========================================================================
// Batched multibin x multistart FdF and L-BFGS
// ===========================================================================
struct pwa_multibin {
	int device = -1, numSMs = 0;
	size_t maxSmem = 0;
	cudaStream_t stream = nullptr;

	struct Bin {
		pwa_likelihood* L;
		LikelihoodView v;
		uint32_t nStarts;
	};
	std::vector<Bin> bins;
	int W = 0, P = 0;
	std::vector<int> slotRe, slotIm;
	int prior = PWA_PRIOR_FLAT;
	double cauchyWidth = 0.5;

	// options
	int SG = 32;
	uint32_t m = 8, maxIter = 5000, floorWindow = 50;
	double gtolAbs = 0., gtolRel = 1e-6;
	uint32_t chunkTiles[3] = {16, 16, 16};  // tiles per work item, by bin size class

	// built state
	bool built = false;
	int Q = 0, nItems = 0;
	DevBuf dBins, dItems, dProblems, dSlotRe, dSlotIm, dPartials, dErr;
	DevBuf dX, dXt, dG, dGt, dD, dF, dFt, dGnorm, dStep, dGamma, dGBest, dS, dY, dRho, dAlpha;
	DevBuf dStatus, dIter, dNBack, dHist, dHead, dItBest, dActive, dNActive;
	PinnedBuf hCount;
	// per check of the last fit: elapsed seconds and every problem's current f
	std::vector<double> traceT, traceF;
	// the device holds a fit state that pwa_multibin_resume can continue
	bool stateValid = false;
	uint32_t sweepsDone = 0;
	// checkpoint file written every checkpointEvery sweeps of a fit (0: none)
	std::string checkpointPath;
	uint32_t checkpointEvery = 0;

	~pwa_multibin()
	{
		if (stream)
			cudaStreamDestroy(stream);
	}
};

namespace {

int sizeClass(uint64_t tiles) { return tiles < 64 ? 0 : (tiles < 512 ? 1 : 2); }

// work items and problem descriptors for the current bins and options
int buildBatch(pwa_multibin* M)
{
	if (M->bins.empty())
		return setError(kErrState, "multibin: no bins added");
	std::vector<BinDesc> bins;
	std::vector<BatchItem> items;
	std::vector<ProblemDesc> problems;
	int q0 = 0;
	for (size_t b = 0; b < M->bins.size(); ++b) {
		const auto& B = M->bins[b];
		BinDesc d{};
		d.amps = B.v.amps;
		d.nEvents = B.v.nEvents;
		d.accI = B.v.accI;
		d.nEvt = B.v.nEvt;
		d.totAcc = B.v.totAcc;
		d.q0 = q0;
		d.nStarts = (int)B.nStarts;
		bins.push_back(d);
		const uint64_t tiles = (B.v.nEvents + 127) / 128;
		const uint32_t chunk = std::max<uint32_t>(1, M->chunkTiles[sizeClass(tiles)]);
		const int groups = ((int)B.nStarts + M->SG - 1) / M->SG;
		for (int g = 0; g < groups; ++g) {
			const int i0 = (int)items.size();
			for (uint64_t t = 0; t < tiles; t += chunk)
				items.push_back(BatchItem{(int)b, g, (uint32_t)t, (uint32_t)std::min<uint64_t>(tiles, t + chunk)});
			const int i1 = (int)items.size();
			for (int s = g * M->SG; s < std::min<int>((int)B.nStarts, (g + 1) * M->SG); ++s)
				problems.push_back(ProblemDesc{(int)b, s - g * M->SG, i0, i1});
		}
		q0 += (int)B.nStarts;
	}
	M->Q = q0;
	M->nItems = (int)items.size();
	PWA_TRY(configureBatchFdf(M->W, M->SG, M->maxSmem));
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	PWA_TRY(M->dBins.alloc(bins.size() * sizeof(BinDesc), "multibin bins"));
	PWA_TRY(M->dItems.alloc(items.size() * sizeof(BatchItem), "multibin items"));
	PWA_TRY(M->dProblems.alloc(problems.size() * sizeof(ProblemDesc), "multibin problems"));
	PWA_TRY(M->dSlotRe.alloc(M->W * sizeof(int), "slot map"));
	PWA_TRY(M->dSlotIm.alloc(M->W * sizeof(int), "slot map"));
	PWA_TRY(M->dPartials.alloc((size_t)M->nItems * M->SG * (2 + 2 * M->W) * sizeof(double), "multibin partials"));
	PWA_TRY(M->dErr.alloc(sizeof(unsigned), "flag"));
	for (DevBuf* b : {&M->dX, &M->dXt, &M->dG, &M->dGt, &M->dD})
		PWA_TRY(b->alloc(Q * P * sizeof(double), "multibin vectors"));
	for (DevBuf* b : {&M->dF, &M->dFt, &M->dGnorm, &M->dStep, &M->dGamma, &M->dGBest})
		PWA_TRY(b->alloc(Q * sizeof(double), "multibin scalars"));
	PWA_TRY(M->dS.alloc(Q * M->m * P * sizeof(double), "L-BFGS history"));
	PWA_TRY(M->dY.alloc(Q * M->m * P * sizeof(double), "L-BFGS history"));
	PWA_TRY(M->dRho.alloc(Q * M->m * sizeof(double), "L-BFGS history"));
	PWA_TRY(M->dAlpha.alloc(Q * M->m * sizeof(double), "L-BFGS history"));
	for (DevBuf* b : {&M->dStatus, &M->dIter, &M->dNBack, &M->dHist, &M->dHead, &M->dItBest, &M->dActive})
		PWA_TRY(b->alloc(Q * sizeof(int), "multibin state"));
	PWA_TRY(M->dNActive.alloc(sizeof(unsigned), "counter"));
	PWA_TRY(M->hCount.ensure(sizeof(unsigned), "counter"));
	cudaStream_t s = M->stream;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dBins.p, bins.data(), bins.size() * sizeof(BinDesc), cudaMemcpyHostToDevice, s),
	                  "upload"));
	PWA_TRY(cudaCheck(
	    cudaMemcpyAsync(M->dItems.p, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, s),
	    "upload"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dProblems.p, problems.data(), problems.size() * sizeof(ProblemDesc),
	                                  cudaMemcpyHostToDevice, s),
	                  "upload"));
	PWA_TRY(cudaCheck(
	    cudaMemcpyAsync(M->dSlotRe.p, M->slotRe.data(), M->W * sizeof(int), cudaMemcpyHostToDevice, s), "upload"));
	PWA_TRY(cudaCheck(
	    cudaMemcpyAsync(M->dSlotIm.p, M->slotIm.data(), M->W * sizeof(int), cudaMemcpyHostToDevice, s), "upload"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "multibin build"));
	M->built = true;
	return kOk;
}

// one evaluation sweep at the trial points dXt of the active problems
int batchSweep(pwa_multibin* M)
{
	BatchArgs a{};
	a.bins = M->dBins.as<BinDesc>();
	a.items = M->dItems.as<BatchItem>();
	a.nItems = M->nItems;
	a.W = M->W;
	a.P = M->P;
	a.SG = M->SG;
	a.slotRe = M->dSlotRe.as<int>();
	a.slotIm = M->dSlotIm.as<int>();
	a.x = M->dXt.as<double>();
	a.active = M->dActive.as<int>();
	a.partials = M->dPartials.as<double>();
	a.devErr = M->dErr.as<unsigned>();
	PWA_TRY(launchBatchFdf(a, M->numSMs, M->stream));
	FinishBatchArgs f{};
	f.bins = a.bins;
	f.problems = M->dProblems.as<ProblemDesc>();
	f.Q = M->Q;
	f.W = M->W;
	f.P = M->P;
	f.SG = M->SG;
	f.slotRe = a.slotRe;
	f.slotIm = a.slotIm;
	f.x = a.x;
	f.active = a.active;
	f.partials = a.partials;
	f.prior = M->prior;
	f.cauchyWidth = M->cauchyWidth;
	f.f = M->dFt.as<double>();
	f.g = M->dGt.as<double>();
	return launchBatchFinish(f, M->stream);
}

LbfgsArgs lbfgsArgs(pwa_multibin* M)
{
	LbfgsArgs l{};
	l.Q = M->Q;
	l.P = M->P;
	l.m = (int)M->m;
	l.maxIter = (int)M->maxIter;
	l.gtolAbs = M->gtolAbs;
	l.gtolRel = M->gtolRel;
	l.x = M->dX.as<double>();
	l.g = M->dG.as<double>();
	l.d = M->dD.as<double>();
	l.xt = M->dXt.as<double>();
	l.ft = M->dFt.as<double>();
	l.gt = M->dGt.as<double>();
	l.f = M->dF.as<double>();
	l.gnorm = M->dGnorm.as<double>();
	l.step = M->dStep.as<double>();
	l.gamma = M->dGamma.as<double>();
	l.gBest = M->dGBest.as<double>();
	l.itBest = M->dItBest.as<int>();
	l.floorWindow = (int)M->floorWindow;
	l.S = M->dS.as<double>();
	l.Y = M->dY.as<double>();
	l.rho = M->dRho.as<double>();
	l.alphaBuf = M->dAlpha.as<double>();
	l.status = M->dStatus.as<int>();
	l.iter = M->dIter.as<int>();
	l.nBack = M->dNBack.as<int>();
	l.hist = M->dHist.as<int>();
	l.head = M->dHead.as<int>();
	return l;
}

int fitSweep(pwa_multibin* M)
{
	PWA_TRY(batchSweep(M));
	PWA_TRY(launchLbfgs(lbfgsArgs(M), M->stream));
	return launchCountActive(M->dStatus.as<int>(), M->Q, M->dActive.as<int>(), M->dNActive.as<unsigned>(),
	                         M->stream);
}

int checkDevErr(pwa_multibin* M)
{
	unsigned e = 0;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(&e, M->dErr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, M->stream), "flag"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(M->stream), "multibin sync"));
	if (e)
		return setError(kErrTimeout, "multibin kernel: a bounded device-side wait expired");
	return kOk;
}

int ensureBuilt(pwa_multibin* M) { return M->built ? kOk : buildBatch(M); }

// uploads trial points and marks every problem active
int startSweep(pwa_multibin* M, const double* x)
{
	M->stateValid = false;  // the trial points and active flags are overwritten
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	cudaStream_t s = M->stream;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dXt.p, x, Q * P * sizeof(double), cudaMemcpyHostToDevice, s), "upload"));
	std::vector<int> ones(Q, 1);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dActive.p, ones.data(), Q * sizeof(int), cudaMemcpyHostToDevice, s), "upload"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(M->dErr.p, 0, sizeof(unsigned), s), "memset"));
	return cudaCheck(cudaStreamSynchronize(s), "upload sync");
}

// The device buffers that hold a batched fit's state, in file order: the
// iterates, trial points, gradients, directions, scalars, L-BFGS histories
// and per-problem counters.  Everything else is rebuilt from the bins.
std::vector<DevBuf*> stateBuffers(pwa_multibin* M)
{
	return {&M->dX,     &M->dXt,    &M->dG,     &M->dGt,    &M->dD,     &M->dF,    &M->dFt,    &M->dGnorm,
	        &M->dStep,  &M->dGamma, &M->dGBest, &M->dS,     &M->dY,     &M->dRho,  &M->dAlpha, &M->dStatus,
	        &M->dIter,  &M->dNBack, &M->dHist,  &M->dHead,  &M->dItBest, &M->dActive};
}

constexpr char kStateMagic[8] = {'R', 'P', 'W', 'A', 'M', 'B', 'S', '1'};

// Checkpoint file: magic, u32 Q, P, m, number of bins, sweeps done, then per
// bin u64 events and u32 starts (checked on load), then every state buffer
// as u64 byte count + bytes.  Written to path + ".tmp" and renamed, so a
// crash while writing leaves the previous checkpoint intact.
int saveState(pwa_multibin* M, const std::string& path)
{
	PWA_TRY(cudaCheck(cudaStreamSynchronize(M->stream), "checkpoint sync"));
	const std::string tmp = path + ".tmp";
	FILE* fp = std::fopen(tmp.c_str(), "wb");
	if (!fp)
		return setError(kErrIo, "cannot create checkpoint '" + tmp + "'");
	bool ok = std::fwrite(kStateMagic, 1, 8, fp) == 8;
	const uint32_t head[5] = {(uint32_t)M->Q, (uint32_t)M->P, M->m, (uint32_t)M->bins.size(), M->sweepsDone};
	ok = ok && std::fwrite(head, sizeof(head), 1, fp) == 1;
	for (const auto& B : M->bins) {
		const uint64_t n = B.v.nEvents;
		ok = ok && std::fwrite(&n, 8, 1, fp) == 1 && std::fwrite(&B.nStarts, 4, 1, fp) == 1;
	}
	std::vector<unsigned char> host;
	int st = kOk;
	for (DevBuf* b : stateBuffers(M)) {
		if (!ok)
			break;
		const uint64_t n = b->bytes;
		host.resize(n);
		st = cudaCheck(cudaMemcpy(host.data(), b->p, n, cudaMemcpyDeviceToHost), "checkpoint download");
		if (st != kOk)
			break;
		ok = std::fwrite(&n, 8, 1, fp) == 1 && std::fwrite(host.data(), 1, n, fp) == n;
	}
	ok = (std::fclose(fp) == 0) && ok;
	if (st != kOk) {
		std::remove(tmp.c_str());
		return st;
	}
	if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
		std::remove(tmp.c_str());
		return setError(kErrIo, "cannot write checkpoint '" + path + "'");
	}
	return kOk;
}

int loadState(pwa_multibin* M, const std::string& path)
{
	FILE* fp = std::fopen(path.c_str(), "rb");
	if (!fp)
		return setError(kErrIo, "cannot open checkpoint '" + path + "'");
	auto fail = [&](const std::string& why) {
		std::fclose(fp);
		return setError(kErrIo, "checkpoint '" + path + "': " + why);
	};
	char magic[8];
	uint32_t head[5];
	if (std::fread(magic, 1, 8, fp) != 8 || std::memcmp(magic, kStateMagic, 8) != 0)
		return fail("not a multibin checkpoint");
	if (std::fread(head, sizeof(head), 1, fp) != 1)
		return fail("truncated header");
	if (head[0] != (uint32_t)M->Q || head[1] != (uint32_t)M->P || head[2] != M->m || head[3] != M->bins.size())
		return fail("problem count, parameter count, history length or bin count differs from this batch");
	for (const auto& B : M->bins) {
		uint64_t n = 0;
		uint32_t starts = 0;
		if (std::fread(&n, 8, 1, fp) != 1 || std::fread(&starts, 4, 1, fp) != 1)
			return fail("truncated bin table");
		if (n != B.v.nEvents || starts != B.nStarts)
			return fail("bin events or starts differ from this batch");
	}
	std::vector<unsigned char> host;
	for (DevBuf* b : stateBuffers(M)) {
		uint64_t n = 0;
		if (std::fread(&n, 8, 1, fp) != 1 || n != b->bytes)
			return fail("state buffer size differs");
		host.resize(n);
		if (std::fread(host.data(), 1, n, fp) != n)
			return fail("truncated state buffer");
		const int st = cudaCheck(cudaMemcpy(b->p, host.data(), n, cudaMemcpyHostToDevice), "checkpoint upload");
		if (st != kOk) {
			std::fclose(fp);
			return st;
		}
	}
	std::fclose(fp);
	M->sweepsDone = head[4];
	M->stateValid = true;
	return kOk;
}

// Runs fit sweeps from the current device state until no problem is active
// or maxSweeps more sweeps have run; writes the checkpoint file between
// graph launches when one is set.
int runFit(pwa_multibin* M, int useGraph, uint32_t sweepsPerGraph, uint32_t maxSweeps, double* x, double* f,
           double* gnorm, int32_t* status, uint32_t* iterations, uint32_t* sweeps)
{
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	cudaStream_t s = M->stream;
	const uint32_t per = std::max<uint32_t>(1, sweepsPerGraph);
	cudaGraphExec_t exec = nullptr;
	if (useGraph) {
		cudaGraph_t g = nullptr;
		PWA_TRY(cudaCheck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture"));
		int st = kOk;
		for (uint32_t i = 0; i < per && st == kOk; ++i)
			st = fitSweep(M);
		const cudaError_t ce = cudaStreamEndCapture(s, &g);
		if (st != kOk) {
			if (g)
				cudaGraphDestroy(g);
			return st;
		}
		PWA_TRY(cudaCheck(ce, "end capture"));
		const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
		cudaGraphDestroy(g);
		PWA_TRY(cudaCheck(ie, "graph instantiate"));
	}
	uint32_t done = 0, lastCheckpoint = M->sweepsDone;
	unsigned* nAct = static_cast<unsigned*>(M->hCount.p);
	int st = kOk;
	M->traceT.clear();
	M->traceF.clear();
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "fit start"));
	const double t0 = seconds();
	while (done < maxSweeps) {
		if (exec)
			st = cudaCheck(cudaGraphLaunch(exec, s), "graph launch");
		else
			for (uint32_t i = 0; i < per && st == kOk; ++i)
				st = fitSweep(M);
		if (st != kOk)
			break;
		done += per;
		M->sweepsDone += per;
		st = cudaCheck(cudaMemcpyAsync(nAct, M->dNActive.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "count");
		if (st == kOk)
			st = cudaCheck(cudaStreamSynchronize(s), "fit sync");
		if (st == kOk) {
			// trace: elapsed time and the accepted f of every problem
			M->traceT.push_back(seconds() - t0);
			const size_t o = M->traceF.size();
			M->traceF.resize(o + Q);
			st = cudaCheck(cudaMemcpy(M->traceF.data() + o, M->dF.p, Q * sizeof(double), cudaMemcpyDeviceToHost),
			               "trace");
		}
		if (st == kOk && M->checkpointEvery > 0 && M->sweepsDone - lastCheckpoint >= M->checkpointEvery) {
			st = saveState(M, M->checkpointPath);
			lastCheckpoint = M->sweepsDone;
		}
		if (st != kOk || *nAct == 0)
			break;
	}
	if (exec)
		cudaGraphExecDestroy(exec);
	PWA_TRY(st);
	if (sweeps)
		*sweeps = done;
	if (x)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(x, M->dX.p, Q * P * sizeof(double), cudaMemcpyDeviceToHost, s), "download"));
	if (f)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(f, M->dF.p, Q * sizeof(double), cudaMemcpyDeviceToHost, s), "download"));
	if (gnorm)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(gnorm, M->dGnorm.p, Q * sizeof(double), cudaMemcpyDeviceToHost, s),
		                  "download"));
	if (status)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(status, M->dStatus.p, Q * sizeof(int), cudaMemcpyDeviceToHost, s),
		                  "download"));
	std::vector<int> it(Q);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(it.data(), M->dIter.p, Q * sizeof(int), cudaMemcpyDeviceToHost, s), "download"));
	PWA_TRY(checkDevErr(M));
	if (iterations)
		for (size_t q = 0; q < Q; ++q)
			iterations[q] = (uint32_t)it[q];
	return kOk;
}

// Times one evaluation sweep (all problems active) in milliseconds.
int timeSweep(pwa_multibin* M, int reps, float* ms)
{
	cudaEvent_t e0, e1;
	PWA_TRY(cudaCheck(cudaEventCreate(&e0), "event"));
	PWA_TRY(cudaCheck(cudaEventCreate(&e1), "event"));
	int st = batchSweep(M);
	cudaEventRecord(e0, M->stream);
	for (int r = 0; r < reps && st == kOk; ++r)
		st = batchSweep(M);
	cudaEventRecord(e1, M->stream);
	if (st == kOk)
		st = cudaCheck(cudaEventSynchronize(e1), "sync");
	if (st == kOk) {
		cudaEventElapsedTime(ms, e0, e1);
		*ms /= (float)reps;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	PWA_TRY(st);
	return checkDevErr(M);
}

}  // namespace

extern "C" {

int pwa_multibin_create(pwa_multibin** out)
{
	if (!out)
		return setError(kErrArg, "null output pointer");
	*out = new pwa_multibin();
	return kOk;
}

int pwa_multibin_destroy(pwa_multibin* M)
{
	delete M;
	return kOk;
}

int pwa_multibin_add_bin(pwa_multibin* M, pwa_likelihood* L, uint32_t nStarts)
{
	if (!M || !L)
		return setError(kErrArg, "null handle");
	if (nStarts == 0)
		return setError(kErrArg, "multibin: a bin needs at least one start point");
	LikelihoodView v;
	PWA_TRY(likelihoodView(L, &v));
	if (v.R != 1 || v.W0 != 0)
		return setError(kErrUnsupported, "multibin batches support rank 1 with one reflectivity");
	if (v.storeB != 128 || v.W > 64)
		return setError(kErrUnsupported, "multibin batches support up to 64 waves");
	if (M->bins.empty()) {
		M->W = v.W;
		M->P = v.P;
		M->slotRe = v.slotRe;
		M->slotIm = v.slotIm;
		M->prior = v.prior;
		M->cauchyWidth = v.cauchyWidth;
		PWA_TRY(deviceInfo(&M->device, &M->numSMs, &M->maxSmem));
		PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking), "stream"));
	} else if (v.W != M->W || v.P != M->P || v.slotRe != M->slotRe || v.slotIm != M->slotIm ||
	           v.prior != M->prior || v.cauchyWidth != M->cauchyWidth) {
		return setError(kErrArg, "multibin: every bin needs the same wave set, parameter layout and prior");
	}
	M->bins.push_back(pwa_multibin::Bin{L, v, nStarts});
	M->built = false;
	M->stateValid = false;
	return kOk;
}

int pwa_multibin_set_options(pwa_multibin* M, uint32_t startGroup, uint32_t lbfgsMemory, double gtolAbs,
                             double gtolRel, uint32_t maxIter)
{
	if (!M)
		return setError(kErrArg, "null handle");
	if (startGroup != 8 && startGroup != 32)
		return setError(kErrArg, "multibin: start group must be 8 or 32");
	if (lbfgsMemory < 1 || lbfgsMemory > 64)
		return setError(kErrArg, "multibin: L-BFGS memory must be 1..64");
	M->SG = (int)startGroup;
	M->m = lbfgsMemory;
	M->gtolAbs = gtolAbs;
	M->gtolRel = gtolRel;
	M->maxIter = maxIter;
	M->built = false;
	M->stateValid = false;
	return kOk;
}

int pwa_multibin_trace(const pwa_multibin* M, uint32_t maxChecks, double* seconds, double* f, uint32_t* nChecks)
{
	if (!M || !nChecks)
		return setError(kErrArg, "null argument");
	const size_t n = M->traceT.size();
	*nChecks = (uint32_t)n;
	const size_t k = std::min<size_t>(n, maxChecks);
	if (seconds)
		std::copy(M->traceT.begin(), M->traceT.begin() + k, seconds);
	if (f && M->Q > 0)
		std::copy(M->traceF.begin(), M->traceF.begin() + k * (size_t)M->Q, f);
	return kOk;
}

int pwa_multibin_set_floor_window(pwa_multibin* M, uint32_t iterations)
{
	if (!M)
		return setError(kErrArg, "null handle");
	M->floorWindow = iterations;
	return kOk;
}

int pwa_multibin_set_chunks(pwa_multibin* M, const uint32_t* tilesPerItem)
{
	if (!M || !tilesPerItem)
		return setError(kErrArg, "null argument");
	for (int c = 0; c < 3; ++c)
		if (tilesPerItem[c] < 1)
			return setError(kErrArg, "multibin: tiles per item must be positive");
	for (int c = 0; c < 3; ++c)
		M->chunkTiles[c] = tilesPerItem[c];
	M->built = false;
	M->stateValid = false;
	return kOk;
}

int pwa_multibin_chunks(const pwa_multibin* M, uint32_t* tilesPerItem)
{
	if (!M || !tilesPerItem)
		return setError(kErrArg, "null argument");
	for (int c = 0; c < 3; ++c)
		tilesPerItem[c] = M->chunkTiles[c];
	return kOk;
}

int pwa_multibin_nmb_problems(const pwa_multibin* M, uint32_t* Q)
{
	if (!M || !Q)
		return setError(kErrArg, "null argument");
	uint32_t q = 0;
	for (const auto& b : M->bins)
		q += b.nStarts;
	*Q = q;
	return kOk;
}

int pwa_multibin_nmb_pars(const pwa_multibin* M, uint32_t* P)
{
	if (!M || !P)
		return setError(kErrArg, "null argument");
	*P = (uint32_t)M->P;
	return kOk;
}

int pwa_multibin_fdf(pwa_multibin* M, const double* x, double* f, double* grad)
{
	if (!M || !x || !f)
		return setError(kErrArg, "null argument");
	PWA_TRY(ensureBuilt(M));
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	cudaStream_t s = M->stream;
	PWA_TRY(startSweep(M, x));
	PWA_TRY(batchSweep(M));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(f, M->dFt.p, Q * sizeof(double), cudaMemcpyDeviceToHost, s), "download"));
	if (grad)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(grad, M->dGt.p, Q * P * sizeof(double), cudaMemcpyDeviceToHost, s),
		                  "download"));
	return checkDevErr(M);
}

int pwa_multibin_sweep_ms(pwa_multibin* M, const double* x, uint32_t reps, double* ms)
{
	if (!M || !x || !ms)
		return setError(kErrArg, "null argument");
	PWA_TRY(ensureBuilt(M));
	PWA_TRY(startSweep(M, x));
	float t = 0.f;
	PWA_TRY(timeSweep(M, (int)std::max<uint32_t>(1, reps), &t));
	*ms = t;
	return kOk;
}

int pwa_multibin_autotune(pwa_multibin* M, const double* x)
{
	if (!M || !x)
		return setError(kErrArg, "null argument");
	static const uint32_t cand[] = {4, 8, 16, 32, 64};
	PWA_TRY(ensureBuilt(M));
	for (int c = 0; c < 3; ++c) {
		uint32_t best = M->chunkTiles[c];
		float bestMs = 1e30f;
		for (uint32_t t : cand) {
			M->chunkTiles[c] = t;
			M->built = false;
			M->stateValid = false;
			PWA_TRY(ensureBuilt(M));
			PWA_TRY(startSweep(M, x));
			float ms = 0.f;
			PWA_TRY(timeSweep(M, 2, &ms));
			if (ms < bestMs) {
				bestMs = ms;
				best = t;
			}
		}
		M->chunkTiles[c] = best;
		M->built = false;
		M->stateValid = false;
	}
	return ensureBuilt(M);
}

int pwa_multibin_fit(pwa_multibin* M, const double* x0, int useGraph, uint32_t sweepsPerGraph, uint32_t maxSweeps,
                     double* x, double* f, double* gnorm, int32_t* status, uint32_t* iterations, uint32_t* sweeps)
{
	if (!M || !x0)
		return setError(kErrArg, "null argument");
	PWA_TRY(ensureBuilt(M));
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	cudaStream_t s = M->stream;
	M->stateValid = false;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dX.p, x0, Q * P * sizeof(double), cudaMemcpyHostToDevice, s), "upload"));
	for (DevBuf* b : {&M->dStatus, &M->dIter, &M->dNBack, &M->dHist, &M->dHead, &M->dItBest})
		PWA_TRY(cudaCheck(cudaMemsetAsync(b->p, 0, Q * sizeof(int), s), "memset"));
	PWA_TRY(startSweep(M, x0));
	M->sweepsDone = 0;
	M->stateValid = true;
	return runFit(M, useGraph, sweepsPerGraph, maxSweeps, x, f, gnorm, status, iterations, sweeps);
}

int pwa_multibin_resume(pwa_multibin* M, int useGraph, uint32_t sweepsPerGraph, uint32_t maxSweeps, double* x,
                        double* f, double* gnorm, int32_t* status, uint32_t* iterations, uint32_t* sweeps)
{
	if (!M)
		return setError(kErrArg, "null argument");
	if (!M->built || !M->stateValid)
		return setError(kErrState, "multibin: no fit state to resume (run a fit or load a saved state first)");
	PWA_TRY(cudaCheck(cudaMemsetAsync(M->dErr.p, 0, sizeof(unsigned), M->stream), "memset"));
	return runFit(M, useGraph, sweepsPerGraph, maxSweeps, x, f, gnorm, status, iterations, sweeps);
}

int pwa_multibin_set_checkpoint(pwa_multibin* M, const char* path, uint32_t everySweeps)
{
	if (!M)
		return setError(kErrArg, "null argument");
	if (everySweeps > 0 && (!path || !*path))
		return setError(kErrArg, "multibin: checkpoint path missing");
	M->checkpointPath = everySweeps > 0 ? path : "";
	M->checkpointEvery = everySweeps;
	return kOk;
}

int pwa_multibin_save_state(pwa_multibin* M, const char* path)
{
	if (!M || !path)
		return setError(kErrArg, "null argument");
	if (!M->built || !M->stateValid)
		return setError(kErrState, "multibin: no fit state to save");
	return saveState(M, path);
}

int pwa_multibin_load_state(pwa_multibin* M, const char* path)
{
	if (!M || !path)
		return setError(kErrArg, "null argument");
	PWA_TRY(ensureBuilt(M));
	return loadState(M, path);
}

int pwa_multibin_sweeps_done(const pwa_multibin* M, uint32_t* sweeps)
{
	if (!M || !sweeps)
		return setError(kErrArg, "null argument");
	*sweeps = M->stateValid ? M->sweepsDone : 0;
	return kOk;
}

}  // extern "C"

// ===========================================================================
// Warm-start network (3-layer perceptron, BF16 with FP32 accumulation)
// ===========================================================================
struct pwa_mlp {
	int nIn = 0, h1 = 0, h2 = 0, nOut = 0;
	size_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0, nPar = 0;
	cudaStream_t stream = nullptr;
	DevBuf params, grads, adamM, adamV, w16;
	// per-batch buffers (capacity cap rows)
	int cap = 0;
	DevBuf x16, h1b, h2b, y32, t32, dy32, dy16, dh16, dh1, dh32, loss, idx;
	// training set on the device
	DevBuf trainX, trainT;
	long step = 0;

	~pwa_mlp()
	{
		if (stream)
			cudaStreamDestroy(stream);
	}
};

namespace {

int mlpEnsureBatch(pwa_mlp* N, int B)
{
	if (B <= N->cap)
		return kOk;
	const size_t b = (size_t)B;
	const int hmax = std::max(N->h1, N->h2);
	PWA_TRY(N->x16.alloc(b * N->nIn * 2, "MLP input"));
	PWA_TRY(N->h1b.alloc(b * N->h1 * 2, "MLP activations"));
	PWA_TRY(N->h2b.alloc(b * N->h2 * 2, "MLP activations"));
	PWA_TRY(N->y32.alloc(b * N->nOut * 4, "MLP output"));
	PWA_TRY(N->t32.alloc(b * N->nOut * 4, "MLP targets"));
	PWA_TRY(N->dy32.alloc(b * N->nOut * 4, "MLP output gradient"));
	PWA_TRY(N->dy16.alloc(b * N->nOut * 2, "MLP output gradient"));
	PWA_TRY(N->dh16.alloc(b * N->h2 * 2, "MLP hidden gradient"));
	PWA_TRY(N->dh1.alloc(b * N->h1 * 2, "MLP hidden gradient"));
	PWA_TRY(N->dh32.alloc(b * hmax * 4, "MLP hidden gradient"));
	PWA_TRY(N->idx.alloc(b * 4, "MLP batch index"));
	PWA_TRY(N->loss.alloc(sizeof(double), "MLP loss"));
	N->cap = B;
	return kOk;
}

MlpGemm gemmXWt(int M, int N, int K, const uint16_t* X, const uint16_t* W)
{
	// C[m][n] = sum_k X[m][k] W[n][k]
	MlpGemm g{};
	g.M = M;
	g.N = N;
	g.K = K;
	g.A = X;
	g.lda_m = (size_t)K;
	g.lda_k = 1;
	g.aContigK = 1;
	g.B = W;
	g.ldb_k = 1;
	g.ldb_n = (size_t)K;
	g.bContigK = 1;
	return g;
}

// forward of a batch already in x16 (B rows): h1b, h2b (BF16), y32
int mlpForward(pwa_mlp* N, int B)
{
	const float* P = N->params.as<float>();
	const uint16_t* W = N->w16.as<uint16_t>();
	MlpGemm g = gemmXWt(B, N->h1, N->nIn, N->x16.as<uint16_t>(), W + N->oW1);
	g.bias = P + N->ob1;
	g.relu = 1;
	g.C16 = N->h1b.as<uint16_t>();
	PWA_TRY(launchMlpGemm(g, N->stream));
	g = gemmXWt(B, N->h2, N->h1, N->h1b.as<uint16_t>(), W + N->oW2);
	g.bias = P + N->ob2;
	g.relu = 1;
	g.C16 = N->h2b.as<uint16_t>();
	PWA_TRY(launchMlpGemm(g, N->stream));
	g = gemmXWt(B, N->nOut, N->h2, N->h2b.as<uint16_t>(), W + N->oW3);
	g.bias = P + N->ob3;
	g.C32 = N->y32.as<float>();
	return launchMlpGemm(g, N->stream);
}

// gradient of the mean squared error of the batch (targets in t32) into grads
int mlpBackward(pwa_mlp* N, int B)
{
	cudaStream_t s = N->stream;
	const uint16_t* W = N->w16.as<uint16_t>();
	float* G = N->grads.as<float>();
	PWA_TRY(cudaCheck(cudaMemsetAsync(N->loss.p, 0, sizeof(double), s), "memset"));
	const int nY = B * N->nOut;
	PWA_TRY(launchMse(N->y32.as<float>(), N->t32.as<float>(), nY, 1.f / (float)nY, N->dy32.as<float>(),
	                  N->dy16.as<uint16_t>(), N->loss.as<double>(), s));
	// dW3[n][k] = sum_b dY[b][n] h2[b][k]
	MlpGemm g{};
	g.M = N->nOut;
	g.N = N->h2;
	g.K = B;
	g.A = N->dy16.as<uint16_t>();
	g.lda_m = 1;
	g.lda_k = (size_t)N->nOut;
	g.B = N->h2b.as<uint16_t>();
	g.ldb_k = (size_t)N->h2;
	g.ldb_n = 1;
	g.C32 = G + N->oW3;
	PWA_TRY(launchMlpGemm(g, s));
	PWA_TRY(launchColSum(N->dy32.as<float>(), B, N->nOut, G + N->ob3, s));
	// dh2 = (dY W3) masked by h2 > 0
	g = MlpGemm{};
	g.M = B;
	g.N = N->h2;
	g.K = N->nOut;
	g.A = N->dy16.as<uint16_t>();
	g.lda_m = (size_t)N->nOut;
	g.lda_k = 1;
	g.aContigK = 1;
	g.B = W + N->oW3;
	g.ldb_k = (size_t)N->h2;
	g.ldb_n = 1;
	g.mask = N->h2b.as<uint16_t>();
	g.C16 = N->dh16.as<uint16_t>();
	g.C32 = N->dh32.as<float>();
	PWA_TRY(launchMlpGemm(g, s));
	PWA_TRY(launchColSum(N->dh32.as<float>(), B, N->h2, G + N->ob2, s));
	// dW2[n][k] = sum_b dh2[b][n] h1[b][k]
	g = MlpGemm{};
	g.M = N->h2;
	g.N = N->h1;
	g.K = B;
	g.A = N->dh16.as<uint16_t>();
	g.lda_m = 1;
	g.lda_k = (size_t)N->h2;
	g.B = N->h1b.as<uint16_t>();
	g.ldb_k = (size_t)N->h1;
	g.ldb_n = 1;
	g.C32 = G + N->oW2;
	PWA_TRY(launchMlpGemm(g, s));
	// dh1 = (dh2 W2) masked by h1 > 0 (dh32 is reused after its last read)
	g = MlpGemm{};
	g.M = B;
	g.N = N->h1;
	g.K = N->h2;
	g.A = N->dh16.as<uint16_t>();
	g.lda_m = (size_t)N->h2;
	g.lda_k = 1;
	g.aContigK = 1;
	g.B = W + N->oW2;
	g.ldb_k = (size_t)N->h1;
	g.ldb_n = 1;
	g.mask = N->h1b.as<uint16_t>();
	g.C16 = N->dh1.as<uint16_t>();
	g.C32 = N->dh32.as<float>();
	PWA_TRY(launchMlpGemm(g, s));
	PWA_TRY(launchColSum(N->dh32.as<float>(), B, N->h1, G + N->ob1, s));
	// dW1[n][k] = sum_b dh1[b][n] x[b][k]
	g = MlpGemm{};
	g.M = N->h1;
	g.N = N->nIn;
	g.K = B;
	g.A = N->dh1.as<uint16_t>();
	g.lda_m = 1;
	g.lda_k = (size_t)N->h1;
	g.B = N->x16.as<uint16_t>();
	g.ldb_k = (size_t)N->nIn;
	g.ldb_n = 1;
	g.C32 = G + N->oW1;
	return launchMlpGemm(g, s);
}

int mlpAdam(pwa_mlp* N, float lr)
{
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	++N->step;
	const float c1 = 1.f - std::pow(b1, (float)N->step), c2 = 1.f - std::pow(b2, (float)N->step);
	return launchAdam(N->params.as<float>(), N->grads.as<float>(), N->adamM.as<float>(), N->adamV.as<float>(),
	                  N->w16.as<uint16_t>(), N->nPar, lr, b1, b2, eps, c1, c2, N->stream);
}

int mlpUploadBatch(pwa_mlp* N, const float* X, const float* T, int B)
{
	PWA_TRY(mlpEnsureBatch(N, B));
	cudaStream_t s = N->stream;
	DevBuf x32;
	PWA_TRY(x32.alloc((size_t)B * N->nIn * 4, "MLP input staging"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(x32.p, X, (size_t)B * N->nIn * 4, cudaMemcpyHostToDevice, s), "upload"));
	PWA_TRY(launchToBf16(x32.as<float>(), N->x16.as<uint16_t>(), (size_t)B * N->nIn, s));
	if (T)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(N->t32.p, T, (size_t)B * N->nOut * 4, cudaMemcpyHostToDevice, s), "upload"));
	return cudaCheck(cudaStreamSynchronize(s), "MLP upload");
}

}  // namespace

extern "C" {

int pwa_mlp_create(pwa_mlp** out, uint32_t nIn, uint32_t nHidden1, uint32_t nHidden2, uint32_t nOut, uint64_t seed)
{
	if (!out || !nIn || !nHidden1 || !nHidden2 || !nOut)
		return setError(kErrArg, "MLP: null output or empty layer");
	std::unique_ptr<pwa_mlp> N(new pwa_mlp());
	N->nIn = (int)nIn;
	N->h1 = (int)nHidden1;
	N->h2 = (int)nHidden2;
	N->nOut = (int)nOut;
	N->oW1 = 0;
	N->ob1 = N->oW1 + (size_t)nHidden1 * nIn;
	N->oW2 = N->ob1 + nHidden1;
	N->ob2 = N->oW2 + (size_t)nHidden2 * nHidden1;
	N->oW3 = N->ob2 + nHidden2;
	N->ob3 = N->oW3 + (size_t)nOut * nHidden2;
	N->nPar = N->ob3 + nOut;
	PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&N->stream, cudaStreamNonBlocking), "stream"));
	for (DevBuf* b : {&N->params, &N->grads, &N->adamM, &N->adamV})
		PWA_TRY(b->alloc(N->nPar * 4, "MLP parameters"));
	PWA_TRY(N->w16.alloc(N->nPar * 2, "MLP BF16 weights"));
	// He-normal weights (std sqrt(2 / fan_in)), zero biases, from a seeded host RNG
	std::vector<float> p(N->nPar, 0.f);
	std::mt19937_64 rng(seed);
	std::normal_distribution<float> nd(0.f, 1.f);
	auto fill = [&](size_t o, size_t rows, size_t cols) {
		const float sd = std::sqrt(2.f / (float)cols);
		for (size_t i = 0; i < rows * cols; ++i)
			p[o + i] = sd * nd(rng);
	};
	fill(N->oW1, nHidden1, nIn);
	fill(N->oW2, nHidden2, nHidden1);
	fill(N->oW3, nOut, nHidden2);
	PWA_TRY(cudaCheck(cudaMemcpy(N->params.p, p.data(), N->nPar * 4, cudaMemcpyHostToDevice), "upload"));
	PWA_TRY(cudaCheck(cudaMemset(N->adamM.p, 0, N->nPar * 4), "memset"));
	PWA_TRY(cudaCheck(cudaMemset(N->adamV.p, 0, N->nPar * 4), "memset"));
	PWA_TRY(launchToBf16(N->params.as<float>(), N->w16.as<uint16_t>(), N->nPar, N->stream));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(N->stream), "MLP init"));
	*out = N.release();
	return kOk;
}

int pwa_mlp_destroy(pwa_mlp* N)
{
	delete N;
	return kOk;
}

int pwa_mlp_nmb_params(const pwa_mlp* N, uint64_t* n)
{
	if (!N || !n)
		return setError(kErrArg, "null argument");
	*n = N->nPar;
	return kOk;
}

int pwa_mlp_get_params(const pwa_mlp* N, float* out)
{
	if (!N || !out)
		return setError(kErrArg, "null argument");
	PWA_TRY(cudaCheck(cudaMemcpyAsync(out, N->params.p, N->nPar * 4, cudaMemcpyDeviceToHost, N->stream), "download"));
	return cudaCheck(cudaStreamSynchronize(N->stream), "MLP parameters");
}

int pwa_mlp_set_params(pwa_mlp* N, const float* in)
{
	if (!N || !in)
		return setError(kErrArg, "null argument");
	PWA_TRY(cudaCheck(cudaMemcpyAsync(N->params.p, in, N->nPar * 4, cudaMemcpyHostToDevice, N->stream), "upload"));
	PWA_TRY(launchToBf16(N->params.as<float>(), N->w16.as<uint16_t>(), N->nPar, N->stream));
	PWA_TRY(cudaCheck(cudaMemsetAsync(N->adamM.p, 0, N->nPar * 4, N->stream), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(N->adamV.p, 0, N->nPar * 4, N->stream), "memset"));
	N->step = 0;
	return cudaCheck(cudaStreamSynchronize(N->stream), "MLP set");
}

int pwa_mlp_forward(pwa_mlp* N, const float* X, uint32_t B, float* Y)
{
	if (!N || !X || !Y || !B)
		return setError(kErrArg, "null argument or empty batch");
	PWA_TRY(mlpUploadBatch(N, X, nullptr, (int)B));
	PWA_TRY(mlpForward(N, (int)B));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(Y, N->y32.p, (size_t)B * N->nOut * 4, cudaMemcpyDeviceToHost, N->stream),
	                  "download"));
	return cudaCheck(cudaStreamSynchronize(N->stream), "MLP forward");
}

int pwa_mlp_gradient(pwa_mlp* N, const float* X, const float* T, uint32_t B, double* loss, float* grad)
{
	if (!N || !X || !T || !B)
		return setError(kErrArg, "null argument or empty batch");
	PWA_TRY(mlpUploadBatch(N, X, T, (int)B));
	PWA_TRY(mlpForward(N, (int)B));
	PWA_TRY(mlpBackward(N, (int)B));
	if (loss)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(loss, N->loss.p, sizeof(double), cudaMemcpyDeviceToHost, N->stream),
		                  "download"));
	if (grad)
		PWA_TRY(cudaCheck(cudaMemcpyAsync(grad, N->grads.p, N->nPar * 4, cudaMemcpyDeviceToHost, N->stream),
		                  "download"));
	return cudaCheck(cudaStreamSynchronize(N->stream), "MLP gradient");
}

int pwa_mlp_train(pwa_mlp* N, const float* X, const float* T, uint64_t nSamples, uint32_t batch, uint32_t epochs,
                  float lr, uint64_t seed, double* lossHistory)
{
	if (!N || !X || !T || !nSamples || !batch)
		return setError(kErrArg, "null argument or empty training set");
	const int B = (int)std::min<uint64_t>(batch, nSamples);
	PWA_TRY(mlpEnsureBatch(N, B));
	cudaStream_t s = N->stream;
	// training set on the device: inputs as BF16, targets FP32
	PWA_TRY(N->trainX.alloc(nSamples * N->nIn * 2, "MLP training inputs"));
	PWA_TRY(N->trainT.alloc(nSamples * N->nOut * 4, "MLP training targets"));
	{
		const uint64_t chunk = std::max<uint64_t>(1, (64ull << 20) / ((uint64_t)N->nIn * 4));
		DevBuf x32;
		PWA_TRY(x32.alloc(std::min(chunk, nSamples) * N->nIn * 4, "MLP input staging"));
		for (uint64_t r = 0; r < nSamples; r += chunk) {
			const uint64_t n = std::min(chunk, nSamples - r);
			PWA_TRY(cudaCheck(cudaMemcpyAsync(x32.p, X + r * N->nIn, n * N->nIn * 4, cudaMemcpyHostToDevice, s),
			                  "upload"));
			PWA_TRY(launchToBf16(x32.as<float>(), N->trainX.as<uint16_t>() + r * N->nIn, n * N->nIn, s));
			PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "upload"));
		}
	}
	PWA_TRY(cudaCheck(cudaMemcpyAsync(N->trainT.p, T, nSamples * N->nOut * 4, cudaMemcpyHostToDevice, s), "upload"));
	std::vector<uint32_t> perm(nSamples);
	for (uint64_t i = 0; i < nSamples; ++i)
		perm[i] = (uint32_t)i;
	std::mt19937_64 rng(seed);
	DevBuf dPerm;
	PWA_TRY(dPerm.alloc(nSamples * 4, "MLP permutation"));
	const uint64_t steps = nSamples / (uint64_t)B;
	for (uint32_t ep = 0; ep < epochs; ++ep) {
		std::shuffle(perm.begin(), perm.end(), rng);
		PWA_TRY(cudaCheck(cudaMemcpyAsync(dPerm.p, perm.data(), nSamples * 4, cudaMemcpyHostToDevice, s), "upload"));
		double epochLoss = 0.;
		for (uint64_t st = 0; st < steps; ++st) {
			const uint32_t* idx = dPerm.as<uint32_t>() + st * B;
			PWA_TRY(launchGatherRows(N->trainX.p, idx, B, (size_t)N->nIn * 2, N->x16.p, s));
			PWA_TRY(launchGatherRows(N->trainT.p, idx, B, (size_t)N->nOut * 4, N->t32.p, s));
			PWA_TRY(mlpForward(N, B));
			PWA_TRY(mlpBackward(N, B));
			double l = 0.;
			PWA_TRY(cudaCheck(cudaMemcpyAsync(&l, N->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s), "download"));
			PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "MLP step"));
			epochLoss += l;
			PWA_TRY(mlpAdam(N, lr));
		}
		if (lossHistory)
			lossHistory[ep] = epochLoss / (double)std::max<uint64_t>(1, steps);
	}
	N->trainX.release();
	N->trainT.release();
	return cudaCheck(cudaStreamSynchronize(s), "MLP train");
}

}  // extern "C"
