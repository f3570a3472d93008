// host_integral.cpp -- the C ABI of ampIntegralMatrix
// (decayAmplitude/ampIntegralMatrix.cc): wave list, GPU integration (SIMT and
// tensor-core Gram kernels), element access, arithmetic and the ASCII file
// format.

#include "host_common.h"

// ===========================================================================
// ampIntegralMatrix
// ===========================================================================

namespace {

// Sums the GPU Gram kernel for integrate().
int gramOnDevice(GramScratch& sc, uint32_t W, const void* amps, uint64_t nEvents, uint32_t nSub, int ampType,
                 int memory, const std::vector<double>& weightK, uint64_t K, int precision, std::vector<cplx>& out)
{
	int dev, sms;
	size_t smem;
	PWA_TRY(deviceInfo(&dev, &sms, &smem));
	if (sc.dev != dev) {
		sc.reset();
		PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking), "stream"));
		sc.dev = dev;
	}
	cudaStream_t s = sc.stream;

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
	DevBuf dIn, dConv, dW;
	DevBuf &dPart = sc.part, &dOut = sc.out, &dErr = sc.err;
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
	PWA_TRY(dOut.ensure((size_t)W * W * 2 * sizeof(double), "integral output"));
	PWA_TRY(dErr.ensure(sizeof(unsigned), "flag"));
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
		PWA_TRY(dPart.ensure(scratch * sizeof(double), "gram partials"));
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
		PWA_TRY(dPart.ensure((size_t)chunks * W * W * 2 * sizeof(double), "gram partials"));
		PWA_TRY(cudaCheck(cudaMemsetAsync(dPart.p, 0, (size_t)chunks * W * W * 2 * sizeof(double), s), "memset"));
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
	if (lastK > 0 && counter > 0) {
		if (!I->scratch.p)
			I->scratch.p.reset(new (std::nothrow) GramScratch());
		if (!I->scratch.p)
			return setError(kErrOom, "out of host memory");
		PWA_TRY(gramOnDevice(*I->scratch.p, nWaves, amps, nEvents, nSubAmps, ampType, memory, weightK, K, precision,
		                     result));
	} else {
		result.assign((size_t)nWaves * nWaves, cplx(0, 0));
	}
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

// containsWave (ampIntegralMatrix.cc:188-191)
int pwa_integral_contains_wave(const pwa_integral* I, const char* name, int* contains)
{
	if (!I || !name || !contains)
		return setError(kErrArg, "null argument");
	*contains = I->index(name) >= 0 ? 1 : 0;
	return kOk;
}

// hasIdenticalWaveSet (ampIntegralMatrix.cc:633-646) and operator ==
// (ampIntegralMatrix.h:179-195): same wave set, same event count and equal
// raw sums element by element, matched by wave name
int pwa_integral_compare(const pwa_integral* I, const pwa_integral* o, int* identicalWaveSet, int* equal)
{
	if (!I || !o)
		return setError(kErrArg, "null argument");
	const bool same = I->sameWaveSet(*o) && o->sameWaveSet(*I);
	bool eq = same && I->nEvents == o->nEvents;
	for (uint32_t i = 0; eq && i < I->nWaves; ++i) {
		const int oi = o->index(I->names[i]);
		for (uint32_t j = 0; eq && j < I->nWaves; ++j)
			eq = I->sums[(size_t)i * I->nWaves + j] == o->sums[(size_t)oi * o->nWaves + o->index(I->names[j])];
	}
	if (identicalWaveSet)
		*identicalWaveSet = same ? 1 : 0;
	if (equal)
		*equal = eq ? 1 : 0;
	return kOk;
}

// clear (ampIntegralMatrix.cc:93-103): no waves, no events
int pwa_integral_clear(pwa_integral* I)
{
	if (!I)
		return setError(kErrArg, "null argument");
	I->nWaves = 0;
	I->nEvents = 0;
	I->names.clear();
	I->sums.clear();
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

int pwa_gram_device_batch(const void* const* amps, const uint64_t* nEvents, uint32_t nBins, uint32_t nWaves,
                          int precision, double* outGram, double* outSums, void* stream)
{
	if (!amps || !nEvents || !outGram)
		return setError(kErrArg, "pwa_gram_device_batch: null argument");
	if (nWaves == 0 || nWaves > 1024)
		return setError(kErrArg, "pwa_gram_device_batch: nWaves must be in 1..1024");
	const bool tc = (precision == PWA_PRECISION_TF32 || precision == PWA_PRECISION_TF32X3 ||
	                 precision == PWA_PRECISION_BF16X3);
	if (!tc && precision != PWA_PRECISION_FP32)
		return setError(kErrUnsupported, "pwa_gram_device_batch: precision must be PWA_PRECISION_FP32, "
		                                 "PWA_PRECISION_TF32, PWA_PRECISION_TF32X3 or PWA_PRECISION_BF16X3");
	for (uint32_t b = 0; b < nBins; ++b)
		if (!amps[b] || nEvents[b] == 0)
			return setError(kErrArg, "pwa_gram_device_batch: bin " + std::to_string(b) + " has no amplitudes");
	if (nBins == 0)
		return kOk;
	int dev, sms;
	size_t smem;
	PWA_TRY(deviceInfo(&dev, &sms, &smem));
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	const int W = (int)nWaves;
	uint64_t nMax = 0;
	for (uint32_t b = 0; b < nBins; ++b)
		nMax = std::max(nMax, nEvents[b]);
	// partials of the largest bin, reused bin after bin in stream order
	const int tps = (W + 63) / 64;
	const int nTiles = tps * (tps + 1) / 2;
	// SIMT chunks as integrate() takes them, within 256 MiB of FP64 partials
	const uint64_t partialBudget = std::max<uint64_t>(1, (256ull << 20) / ((uint64_t)W * W * 2 * sizeof(double)));
	const int simtChunks = (int)std::min<uint64_t>(
	    std::min<uint64_t>((uint64_t)std::max(1, (4 * sms + nTiles - 1) / nTiles), std::max<uint64_t>(1, nMax / 64)),
	    partialBudget);
	const size_t tcScratch = tc ? gramTcScratchFloats(W, sms) / 2 + 1 : 0;
	// tensor-core precisions: bins whose rows are not 16-byte aligned (odd
	// event count or base) are copied into an aligned buffer of even row
	// length first, reused bin after bin in stream order
	uint64_t nPad = 0;
	if (tc)
		for (uint32_t b = 0; b < nBins; ++b)
			if (nEvents[b] >= 128 && ((nEvents[b] & 1ull) || (reinterpret_cast<uintptr_t>(amps[b]) & 15u)))
				nPad = std::max<uint64_t>(nPad, nEvents[b] + (nEvents[b] & 1ull));
	DevBuf dPart, dErr, dAlign;
	PWA_TRY(dPart.alloc(std::max(tcScratch, (size_t)simtChunks * W * W * 2) * sizeof(double), "gram batch partials"));
	if (nPad)
		PWA_TRY(dAlign.alloc((size_t)W * nPad * sizeof(float2), "gram batch alignment buffer"));
	PWA_TRY(dErr.alloc(sizeof(unsigned), "flag"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dErr.p, 0, sizeof(unsigned), s), "memset"));
	for (uint32_t b = 0; b < nBins; ++b) {
		const uint64_t n = nEvents[b];
		GramArgs g{};
		g.amps = static_cast<const float2*>(amps[b]);
		g.K = n;
		g.ldK = n;
		g.W = W;
		g.devErr = dErr.as<unsigned>();
		double* out = outGram + (size_t)b * W * W * 2;
		if (outSums)
			PWA_TRY(launchRowSums(g.amps, n, n, W, outSums + (size_t)b * W * 2, s));
		// the tensor-core kernel reads rows with TMA: an even row length
		// (16-byte rows) and a 16-byte aligned base; bins shorter than one
		// 128-event box take the SIMT kernel
		int st = kErrUnsupported;
		if (tc && n >= 128) {
			if ((n & 1ull) || (reinterpret_cast<uintptr_t>(amps[b]) & 15u)) {
				const uint64_t ld = n + (n & 1ull);
				PWA_TRY(cudaCheck(cudaMemcpy2DAsync(dAlign.p, ld * sizeof(float2), amps[b], n * sizeof(float2),
				                                    n * sizeof(float2), W, cudaMemcpyDeviceToDevice, s),
				                  "gram batch realignment"));
				g.amps = dAlign.as<float2>();
				g.ldK = ld;
			}
			st = launchGramTc(g, precision, sms, s, out, dPart.as<double>(), tcScratch);
			if (st != kOk && st != kErrUnsupported)
				return st;
		}
		// FP32, or a shape the tensor-core kernel does not take: SIMT kernel
		if (st != kOk) {
			g.amps = static_cast<const float2*>(amps[b]);
			g.ldK = n;
			g.chunks = (int)std::min<uint64_t>((uint64_t)simtChunks, std::max<uint64_t>(1, n / 64));
			g.partials = dPart.as<double>();
			PWA_TRY(launchGramSimt(g, 1, s));
			PWA_TRY(launchGramReduce(g.partials, g.chunks, W, out, 0, s));
		}
	}
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "gram batch"));
	unsigned err = 0;
	PWA_TRY(cudaCheck(cudaMemcpy(&err, dErr.p, sizeof(unsigned), cudaMemcpyDeviceToHost), "flag"));
	if (err)
		return setError(kErrTimeout, "pwa_gram_device_batch: a bounded device-side wait expired");
	return kOk;
}

}  // extern "C"
