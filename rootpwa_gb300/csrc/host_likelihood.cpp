// host_likelihood.cpp -- the C ABI of pwaLikelihood<complex<double>>
// (partialWaveFit/pwaLikelihood.cc): setup (wave list, parameter layout,
// integral reordering and rescaling, amplitude normalisation, on-the-fly
// binning and amplitude files) in FP64 on the host following the reference
// line by line, evaluation through the fused FdF kernels, the Hessian and
// covariance, the autotuner and its cache, and the read-only device view
// that the batched fits use.

#include "host_common.h"

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
	uint32_t storeBRequest = 0;  // pwa_likelihood_set_store_block (0: automatic)
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
	a.active = nullptr;
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
	// the computation proper, timed on the host like the reference's
	// stopwatch (no timing events on the host-call path)
	const double t1 = seconds();
	PWA_TRY(launchEval(L, static_cast<const double*>(L->hPar.dev), static_cast<double*>(L->hOut.dev), withGrad, s));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "FdF sync"));
	const double tFunc = seconds() - t1;
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
	CallInfo& ci = L->info[call];
	++ci.nCalls;
	ci.func += tFunc;  // the fused kernel includes the normalisation term
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

int pwa_likelihood_options(const pwa_likelihood* L, int* useNormalizedAmps, int* priorType, double* cauchyWidth)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (useNormalizedAmps)
		*useNormalizedAmps = L->useNormalizedAmps ? 1 : 0;
	if (priorType)
		*priorType = L->priorType;
	if (cauchyWidth)
		*cauchyWidth = L->cauchyWidth;
	return kOk;
}

int pwa_likelihood_deriv_cache(const pwa_likelihood* L, double* grad)
{
	if (!L || !grad)
		return setError(kErrArg, "null argument");
	if (!L->cacheValid)
		return setError(kErrState, "no gradient evaluated since the last change");
	std::copy(L->derivCache.begin(), L->derivCache.end(), grad);
	return kOk;
}

// clear (pwaLikelihood.cc:1670-1674) releases the decay amplitudes; here the
// device amplitude store.  Evaluation is refused until the amplitudes are
// added and finishInit is called again.
int pwa_likelihood_clear(pwa_likelihood* L)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (L->stream)
		cudaStreamSynchronize(L->stream);
	L->amps.release();
	L->ampTmp.release();
	for (int e = 0; e < 2; ++e)
		std::fill(L->added[e].begin(), L->added[e].end(), 0);
	L->finished = false;
	L->cacheValid = false;
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

int pwa_likelihood_set_store_block(pwa_likelihood* L, uint32_t events)
{
	if (!L)
		return setError(kErrArg, "null likelihood");
	if (events != 0 && events != 64 && events != 128)
		return setError(kErrArg, "store block must be 64 or 128 events (0: automatic)");
	if (L->nEvents != 0)
		return setError(kErrState, "the store block is fixed by the first addAmplitude()");
	L->storeBRequest = events;
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
	if (phase1Events < 0 || phase1Events > 5)
		return setError(kErrArg, "FdF kernel variant must be 1, 2 or 4 (events per lane), 3 (fused gradient), "
		                         "5 (narrow, one event per thread) or 0 (keep)");
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
	if (r != PWA_REDUCE_FP64 && r != PWA_REDUCE_KAHAN_FP32 && r != PWA_REDUCE_FP32)
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
		L->storeB = L->storeBRequest ? L->storeBRequest
		                             : (uint32_t)chooseStoreBlock((int)L->W(), (int)L->rank, L->maxSmem);
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
	// The weighted Grams run on the tensor cores (TF32x3, the hi/lo kernel of
	// gram_tc.cu, up to 96 columns): a set of at most 96 columns in one Gram;
	// a wider set is split into groups of 48 rows, and the Gram of each pair
	// of groups (one 3-D TMA copy brings both) supplies their cross block and
	// the groups' diagonal blocks.  The operand rows are padded with zero rows
	// to whole groups.
	auto groupsOf = [](uint32_t n, uint32_t* G, uint32_t* ng) {
		*G = n <= 96 ? n : 48;
		*ng = (n + *G - 1) / *G;
	};
	uint32_t gs1, ng1, gs2, ng2;
	groupsOf(nY1, &gs1, &ng1);
	groupsOf(nY2, &gs2, &ng2);
	const uint64_t rows1 = (uint64_t)gs1 * ng1, rows2 = (uint64_t)gs2 * ng2;
	// event slabs sized so that the [d; conj d; 1] columns stay below ~4 GB
	// (10^6 events of the 349-column set in one slab: fewer, longer Gram
	// launches); a multiple of 64 events (the tensor maps want an even row
	// stride)
	uint64_t slab = (uint64_t)4 << 30;
	slab /= rows1 * sizeof(float2);
	slab = std::max<uint64_t>(1024, std::min<uint64_t>(slab, (L->nEvents + 63) / 64 * 64)) / 64 * 64;
	const uint32_t maxGram = std::max(ng1 > 1 ? 2 * gs1 : gs1, ng2 > 1 ? 2 * gs2 : gs2);
	const size_t scratch = gramTcScratchFloats((int)maxGram, L->numSMs) / 2 + 1;
	DevBuf dY1, dY2, dW1, dW2, dPart, dBlk, dErrG, dG1, dG2, dHP;
	PWA_TRY(dY1.alloc((size_t)rows1 * slab * sizeof(float2), "hessian operand"));
	PWA_TRY(dY2.alloc((size_t)rows2 * slab * sizeof(float2), "hessian operand"));
	PWA_TRY(dW1.alloc(slab * sizeof(double), "hessian weights"));
	PWA_TRY(dW2.alloc(slab * sizeof(double), "hessian weights"));
	PWA_TRY(dPart.alloc(scratch * sizeof(double), "hessian gram partials"));
	PWA_TRY(dBlk.alloc((size_t)maxGram * maxGram * 2 * sizeof(double), "hessian gram block"));
	PWA_TRY(dErrG.alloc(sizeof(unsigned), "flag"));
	PWA_TRY(dG1.alloc((size_t)nY1 * nY1 * 2 * sizeof(double), "hessian gram"));
	PWA_TRY(dG2.alloc((size_t)nY2 * nY2 * 2 * sizeof(double), "hessian gram"));
	PWA_TRY(dHP.alloc(P * sizeof(double), "hessian parameters"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(dHP.p, par, P * sizeof(double), cudaMemcpyHostToDevice, s), "H2D par"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dG1.p, 0, dG1.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dG2.p, 0, dG2.bytes, s), "memset"));
	PWA_TRY(cudaCheck(cudaMemsetAsync(dErrG.p, 0, sizeof(unsigned), s), "memset"));
	if (rows1 > nY1)
		PWA_TRY(cudaCheck(cudaMemsetAsync(dY1.as<float2>() + (size_t)nY1 * slab, 0,
		                                  (size_t)(rows1 - nY1) * slab * sizeof(float2), s),
		                  "memset"));
	if (rows2 > nY2)
		PWA_TRY(cudaCheck(cudaMemsetAsync(dY2.as<float2>() + (size_t)nY2 * slab, 0,
		                                  (size_t)(rows2 - nY2) * slab * sizeof(float2), s),
		                  "memset"));
	// dG (n x n) += the weighted Gram of the n rows of Y over K events
	auto gramAdd = [&](const float2* Y, uint32_t n, uint32_t G, uint32_t ng, const double* w, uint64_t K,
	                   double* dG) -> int {
		GramArgs g{};
		g.K = K;
		g.ldK = slab;
		g.weightK = w;
		g.devErr = dErrG.as<unsigned>();
		if (ng == 1) {
			g.amps = Y;
			g.W = (int)n;
			PWA_TRY(launchGramTc(g, PWA_PRECISION_TF32X3, L->numSMs, s, dBlk.as<double>(), dPart.as<double>(), scratch));
			return launchGramBlockAdd(dBlk.as<double>(), (int)n, (int)n, 0, 0, (int)n, 1, 1, dG, s);
		}
		for (uint32_t ga = 0; ga < ng; ++ga)
			for (uint32_t gb = ga + 1; gb < ng; ++gb) {
				g.amps = Y + (size_t)ga * G * slab;
				g.W = (int)(2 * G);
				g.groupStride = (uint64_t)(gb - ga) * G * slab;
				PWA_TRY(launchGramTc(g, PWA_PRECISION_TF32X3, L->numSMs, s, dBlk.as<double>(), dPart.as<double>(),
				                     scratch));
				// group ga's diagonal block from its pair with ga + 1, the last
				// group's from the last pair
				PWA_TRY(launchGramBlockAdd(dBlk.as<double>(), (int)(2 * G), (int)G, (int)ga, (int)gb, (int)n,
				                           gb == ga + 1 ? 1 : 0, (ga + 2 == ng && gb + 1 == ng) ? 1 : 0, dG, s));
			}
		return kOk;
	};
	for (uint64_t e0 = 0; e0 < L->nEvents; e0 += slab) {
		const uint64_t K = std::min<uint64_t>(slab, L->nEvents - e0);
		PWA_TRY(launchHessPrep(L->amps.as<float2>(), L->nEvents, L->storeB, e0, slab, (int)L->nW[0], (int)W, (int)R,
		                       (int)P, dHP.as<double>(), L->dSlotRe.as<int>(), L->dSlotIm.as<int>(), dY1.as<float2>(),
		                       dY2.as<float2>(), dW1.as<double>(), dW2.as<double>(), s));
		PWA_TRY(gramAdd(dY1.as<float2>(), nY1, gs1, ng1, dW1.as<double>(), K, dG1.as<double>()));
		PWA_TRY(gramAdd(dY2.as<float2>(), nY2, gs2, ng2, dW2.as<double>(), K, dG2.as<double>()));
	}
	unsigned gramErr = 0;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(&gramErr, dErrG.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "D2H flag"));
	std::vector<double> G1((size_t)nY1 * nY1 * 2), G2((size_t)nY2 * nY2 * 2);
	PWA_TRY(cudaCheck(cudaMemcpyAsync(G1.data(), dG1.p, G1.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(G2.data(), dG2.p, G2.size() * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "hessian sync"));
	if (gramErr)
		return setError(kErrTimeout, "Hessian Gram kernel: a bounded device-side wait expired");
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

// HessianEigenVectors (pwaLikelihood.cc:864-912): eigen-decomposition of the
// Hessian restricted to the free parameters, eigenvectors embedded in the
// full parameter space with zeros at the fixed parameters.  Cyclic Jacobi
// rotations in FP64 on the host (symmetric P x P, once per fit): each
// rotation zeroes one off-diagonal pair; sweeps repeat until the
// off-diagonal sum of squares is below 1e-30 of the total
// (PWA_ERROR_NUMERICAL if 100 sweeps do not get there).  Eigenvalues in
// descending order; the sign of each eigenvector is arbitrary.
int pwa_likelihood_hessian_eigenvectors(const pwa_likelihood* L, const double* H, double* eigenvalues,
                                        double* eigenvectors, uint32_t* nFree)
{
	if (!L || !H || !eigenvalues || !eigenvectors || !nFree)
		return setError(kErrArg, "null argument");
	if (!L->initialized)
		return setError(kErrState, "likelihood not initialized");
	const uint32_t P = L->nPars;
	std::vector<uint32_t> fr;
	for (uint32_t i = 0; i < P; ++i)
		if (!L->pars[i].fixed)
			fr.push_back(i);
	const size_t n = fr.size();
	std::vector<double> a(n * n), v(n * n, 0.);
	double total = 0.;
	for (size_t i = 0; i < n; ++i) {
		for (size_t j = 0; j < n; ++j) {
			// symmetrise: the Hessian is symmetric up to rounding
			const double x = 0.5 * (H[(size_t)fr[i] * P + fr[j]] + H[(size_t)fr[j] * P + fr[i]]);
			a[i * n + j] = x;
			total += x * x;
			if (!std::isfinite(x))
				return setError(kErrNumerical, "Hessian has non-finite entries");
		}
		v[i * n + i] = 1.;
	}
	const int kMaxSweeps = 100;
	bool converged = false;
	for (int sweep = 0; sweep <= kMaxSweeps; ++sweep) {
		double off = 0.;
		for (size_t p = 0; p < n; ++p)
			for (size_t q = p + 1; q < n; ++q)
				off += a[p * n + q] * a[p * n + q];
		if (off <= 1e-30 * total || off == 0.) {
			converged = true;
			break;
		}
		if (sweep == kMaxSweeps)
			break;
		for (size_t p = 0; p < n; ++p)
			for (size_t q = p + 1; q < n; ++q) {
				const double apq = a[p * n + q];
				if (apq == 0.)
					continue;
				// rotation angle that zeroes a_pq: t = tan(phi) is the smaller
				// root of t^2 + 2 theta t - 1 = 0, theta = (a_qq - a_pp) / (2 a_pq)
				const double theta = (a[q * n + q] - a[p * n + p]) / (2. * apq);
				const double t = (theta >= 0. ? 1. : -1.) / (std::fabs(theta) + std::sqrt(theta * theta + 1.));
				const double c = 1. / std::sqrt(t * t + 1.), sn = t * c;
				for (size_t k = 0; k < n; ++k) {  // columns p, q
					const double akp = a[k * n + p], akq = a[k * n + q];
					a[k * n + p] = c * akp - sn * akq;
					a[k * n + q] = sn * akp + c * akq;
				}
				for (size_t k = 0; k < n; ++k) {  // rows p, q
					const double apk = a[p * n + k], aqk = a[q * n + k];
					a[p * n + k] = c * apk - sn * aqk;
					a[q * n + k] = sn * apk + c * aqk;
				}
				for (size_t k = 0; k < n; ++k) {  // eigenvectors as columns of v
					const double vkp = v[k * n + p], vkq = v[k * n + q];
					v[k * n + p] = c * vkp - sn * vkq;
					v[k * n + q] = sn * vkp + c * vkq;
				}
				// the rotation zeroes a_pq; set it exactly instead of keeping
				// its rounding residue, so that the off-diagonal norm can fall
				// below the threshold
				a[p * n + q] = a[q * n + p] = 0.;
			}
	}
	if (!converged)
		return setError(kErrNumerical, "HessianEigenVectors: Jacobi rotations did not converge in " +
		                                   std::to_string(kMaxSweeps) + " sweeps");
	std::vector<size_t> order(n);
	for (size_t i = 0; i < n; ++i)
		order[i] = i;
	std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return a[x * n + x] > a[y * n + y]; });
	std::fill(eigenvalues, eigenvalues + P, 0.);
	std::fill(eigenvectors, eigenvectors + (size_t)P * P, 0.);
	for (size_t k = 0; k < n; ++k) {
		const size_t col = order[k];
		eigenvalues[k] = a[col * n + col];
		for (size_t i = 0; i < n; ++i)
			eigenvectors[k * P + fr[i]] = v[i * n + col];
	}
	*nFree = (uint32_t)n;
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

int launchLikelihoodEval(pwa_likelihood* L, const double* dPar, double* dOut, const int* dActive, cudaStream_t s)
{
	PWA_TRY(checkFinished(L));
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
	a.withGrad = 1;
	a.reduction = L->reduction;
	a.nPartial = 2 + 2 * a.R * a.W;
	a.fixAcc = L->dFixAcc.as<unsigned long long>();
	a.nfAcc = L->dNfAcc.as<double>();
	a.counter = L->dCounter.as<unsigned>();
	a.devErr = L->dErr.as<unsigned>();
	a.out = dOut;
	a.active = dActive;
	return launchFdf(L->plan, a, s);
}

int clearLikelihoodError(pwa_likelihood* L, cudaStream_t s)
{
	PWA_TRY(checkFinished(L));
	return cudaCheck(cudaMemsetAsync(L->dErr.p, 0, sizeof(unsigned), s), "clear device error flag");
}

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
	v->fixed.assign(L->nPars, 0);
	for (uint32_t i = 0; i < L->nPars; ++i)
		v->fixed[i] = L->pars[i].fixed ? 1 : 0;
	return kOk;
}

}  // namespace pwa
