// host_mlp.cpp -- the warm-start network: parameters, forward and backward
// passes and Adam training over the kernels of mlp.cu.

#include "host_common.h"

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
	// K-slice partials of the tensor-core GEMMs
	int numSMs = 1;
	DevBuf work;
	size_t workFloats = 0;
	DevBuf dErr;  // device error flag of the GEMM kernel's bounded waits

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

// one product on the tensor cores, split over K so that its blocks cover
// the GPU; the workspace of the K-slice partials grows to the largest product
// on first use (a batch size's first step)
int mlpGemm(pwa_mlp* N, MlpGemm g, cudaStream_t s)
{
	g.splitK = mlpGemmSplit(g, N->numSMs);
	const size_t need = (size_t)g.splitK * g.M * g.N;
	if (need > N->workFloats) {
		PWA_TRY(N->work.alloc(need * sizeof(float), "MLP K-slice workspace"));
		N->workFloats = need;
	}
	g.work = N->work.as<float>();
	g.devErr = N->dErr.as<unsigned>();
	return launchMlpGemm(g, s);
}

// after a synchronisation: a bounded wait of a GEMM kernel expired?
int mlpCheckDevice(pwa_mlp* N)
{
	unsigned e = 0;
	PWA_TRY(cudaCheck(cudaMemcpy(&e, N->dErr.p, sizeof(unsigned), cudaMemcpyDeviceToHost), "MLP error flag"));
	if (e) {
		cudaMemset(N->dErr.p, 0, sizeof(unsigned));
		return setError(kErrTimeout, "MLP GEMM kernel: a bounded device-side wait expired");
	}
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
	PWA_TRY(mlpGemm(N, g, N->stream));
	g = gemmXWt(B, N->h2, N->h1, N->h1b.as<uint16_t>(), W + N->oW2);
	g.bias = P + N->ob2;
	g.relu = 1;
	g.C16 = N->h2b.as<uint16_t>();
	PWA_TRY(mlpGemm(N, g, N->stream));
	g = gemmXWt(B, N->nOut, N->h2, N->h2b.as<uint16_t>(), W + N->oW3);
	g.bias = P + N->ob3;
	g.C32 = N->y32.as<float>();
	return mlpGemm(N, g, N->stream);
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
	PWA_TRY(mlpGemm(N, g, s));
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
	PWA_TRY(mlpGemm(N, g, s));
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
	PWA_TRY(mlpGemm(N, g, s));
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
	PWA_TRY(mlpGemm(N, g, s));
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
	return mlpGemm(N, g, s);
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
	int dev = 0;
	PWA_TRY(cudaCheck(cudaGetDevice(&dev), "cudaGetDevice"));
	PWA_TRY(cudaCheck(cudaDeviceGetAttribute(&N->numSMs, cudaDevAttrMultiProcessorCount, dev), "SM count"));
	for (DevBuf* b : {&N->params, &N->grads, &N->adamM, &N->adamV})
		PWA_TRY(b->alloc(N->nPar * 4, "MLP parameters"));
	PWA_TRY(N->w16.alloc(N->nPar * 2, "MLP BF16 weights"));
	PWA_TRY(N->dErr.alloc(sizeof(unsigned), "MLP error flag"));
	PWA_TRY(cudaCheck(cudaMemset(N->dErr.p, 0, sizeof(unsigned)), "memset"));
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
	PWA_TRY(cudaCheck(cudaStreamSynchronize(N->stream), "MLP forward"));
	return mlpCheckDevice(N);
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
	PWA_TRY(cudaCheck(cudaStreamSynchronize(N->stream), "MLP gradient"));
	return mlpCheckDevice(N);
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
		PWA_TRY(mlpCheckDevice(N));
	}
	N->trainX.release();
	N->trainT.release();
	return cudaCheck(cudaStreamSynchronize(s), "MLP train");
}

}  // extern "C"
