// host_multibin.cpp -- batched multibin x multistart fits: work items over
// the bins' amplitude stores, graph-captured sweeps of the batched FdF and
// L-BFGS kernels, the chunk autotuner and checkpoint / resume of the fit
// state.  Bins of rank 1 with one reflectivity and at most 64 waves run the
// start-packed batch kernels; every other layout of the reference (any rank,
// both reflectivities, up to the FdF kernel's wave limit) evaluates each
// (bin, start) problem with its bin's own FdF kernel inside the same
// captured sweep.  Parameters the layout holds fixed (threshold-fixed and
// all-zero waves) start at 0 and keep a zero gradient, as the reference's
// minimiser drivers keep them at 0 (pwaFit.cc:249-266,
// pwaNloptFit.cc:383-401).

#include "host_common.h"

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
	// general layout: one FdF launch of the bin's own kernel per problem
	bool general = false;
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
	DevBuf dFixed;   // [bins][P] fixed-parameter masks
	DevBuf dOut;     // general layout: [Q][P + 2] FdF outputs
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
		if (M->general) {
			for (uint32_t s = 0; s < B.nStarts; ++s)
				problems.push_back(ProblemDesc{(int)b, (int)s, 0, 0});
			q0 += (int)B.nStarts;
			continue;
		}
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
	const size_t Q = (size_t)M->Q, P = (size_t)M->P;
	std::vector<unsigned char> fixed;
	for (const auto& B : M->bins)
		fixed.insert(fixed.end(), B.v.fixed.begin(), B.v.fixed.end());
	PWA_TRY(M->dFixed.alloc(fixed.size(), "multibin fixed masks"));
	PWA_TRY(M->dBins.alloc(bins.size() * sizeof(BinDesc), "multibin bins"));
	PWA_TRY(M->dProblems.alloc(problems.size() * sizeof(ProblemDesc), "multibin problems"));
	if (M->general) {
		PWA_TRY(M->dOut.alloc(Q * (P + 2) * sizeof(double), "multibin FdF outputs"));
	} else {
		PWA_TRY(configureBatchFdf(M->W, M->SG, M->maxSmem));
		PWA_TRY(M->dItems.alloc(items.size() * sizeof(BatchItem), "multibin items"));
		PWA_TRY(M->dSlotRe.alloc(M->W * sizeof(int), "slot map"));
		PWA_TRY(M->dSlotIm.alloc(M->W * sizeof(int), "slot map"));
		PWA_TRY(M->dPartials.alloc((size_t)M->nItems * M->SG * (2 + 2 * M->W) * sizeof(double),
		                           "multibin partials"));
	}
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
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dProblems.p, problems.data(), problems.size() * sizeof(ProblemDesc),
	                                  cudaMemcpyHostToDevice, s),
	                  "upload"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dFixed.p, fixed.data(), fixed.size(), cudaMemcpyHostToDevice, s), "upload"));
	if (!M->general) {
		PWA_TRY(cudaCheck(
		    cudaMemcpyAsync(M->dItems.p, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, s),
		    "upload"));
		PWA_TRY(cudaCheck(
		    cudaMemcpyAsync(M->dSlotRe.p, M->slotRe.data(), M->W * sizeof(int), cudaMemcpyHostToDevice, s), "upload"));
		PWA_TRY(cudaCheck(
		    cudaMemcpyAsync(M->dSlotIm.p, M->slotIm.data(), M->W * sizeof(int), cudaMemcpyHostToDevice, s), "upload"));
	}
	PWA_TRY(cudaCheck(cudaStreamSynchronize(s), "multibin build"));
	M->built = true;
	return kOk;
}

// one evaluation sweep at the trial points dXt of the active problems
int batchSweep(pwa_multibin* M)
{
	if (M->general) {
		const size_t P = (size_t)M->P;
		int q = 0;
		for (const auto& B : M->bins)
			for (uint32_t s = 0; s < B.nStarts; ++s, ++q)
				PWA_TRY(launchLikelihoodEval(B.L, M->dXt.as<double>() + q * P, M->dOut.as<double>() + q * (P + 2),
				                             M->dActive.as<int>() + q, M->stream));
		GatherEvalArgs g{};
		g.Q = M->Q;
		g.P = M->P;
		g.out = M->dOut.as<double>();
		g.active = M->dActive.as<int>();
		g.problems = M->dProblems.as<ProblemDesc>();
		g.fixed = M->dFixed.as<unsigned char>();
		g.f = M->dFt.as<double>();
		g.g = M->dGt.as<double>();
		g.devErr = M->dErr.as<unsigned>();
		return launchGatherEval(g, M->stream);
	}
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
	f.fixed = M->dFixed.as<unsigned char>();
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
	if (M->general)
		for (const auto& B : M->bins)
			PWA_TRY(clearLikelihoodError(B.L, s));
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
	// the start-packed kernels: rank 1, one reflectivity, <= 64 waves,
	// 128-event store blocks; anything else is batched with the bins' own
	// FdF kernels
	const bool general = !(v.R == 1 && v.W0 == 0 && v.storeB == 128 && v.W <= 64);
	if (M->bins.empty()) {
		M->general = general;
		M->W = v.W;
		M->P = v.P;
		M->slotRe = v.slotRe;
		M->slotIm = v.slotIm;
		M->prior = v.prior;
		M->cauchyWidth = v.cauchyWidth;
		PWA_TRY(deviceInfo(&M->device, &M->numSMs, &M->maxSmem));
		PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking), "stream"));
	} else if (general != M->general || v.W != M->W || v.P != M->P || v.slotRe != M->slotRe ||
	           v.slotIm != M->slotIm || v.prior != M->prior || v.cauchyWidth != M->cauchyWidth) {
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
	if (M->general)
		return kOk;  // each bin's FdF plan was tuned by its likelihood
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
	// parameters held fixed start (and stay) at 0
	std::vector<double> start(x0, x0 + Q * P);
	size_t q = 0;
	for (const auto& B : M->bins)
		for (uint32_t k = 0; k < B.nStarts; ++k, ++q)
			for (size_t i = 0; i < P; ++i)
				if (B.v.fixed[i])
					start[q * P + i] = 0.;
	PWA_TRY(cudaCheck(cudaMemcpyAsync(M->dX.p, start.data(), Q * P * sizeof(double), cudaMemcpyHostToDevice, s),
	                  "upload"));
	for (DevBuf* b : {&M->dStatus, &M->dIter, &M->dNBack, &M->dHist, &M->dHead, &M->dItBest})
		PWA_TRY(cudaCheck(cudaMemsetAsync(b->p, 0, Q * sizeof(int), s), "memset"));
	PWA_TRY(startSweep(M, start.data()));
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
