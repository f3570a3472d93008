// host_isobar.cpp -- C ABI of the three-body isobar decay amplitudes: the
// wave set, the final state, the options of isobarAmplitude
// (decayAmplitude/isobarAmplitude.h:68-75) and the evaluation on the GPU
// (isobar.cu); the spin-algebra utilities the plan is built from.
#include "host_common.h"
#include "isobar_plan.h"

#include <fcntl.h>
#include <unistd.h>

struct pwa_isobar {
	double masses[3] = {0.0, 0.0, 0.0};
	int32_t species[3] = {0, 1, 2};
	double beamMass = 0.0;
	bool finalState = false;
	bool reflBasis = true, bose = true, spaceInversion = false, reflection = false, canonical = false;
	bool isospinSet = false, isospinSym = false;
	uint64_t chunkEvents = 0;  // host-buffer calls: events per device pass (0: 1 GiB of buffers)
	iso::FsIsospin isospin{};
	std::vector<pwa_isobar_wave> waves;
	iso::Plan plan;
	bool dirty = true;
	DevBuf dPlan, dIn, dOut;
	iso::PlanView devView{};
	cudaStream_t stream = nullptr;
	bool ownStream = false;   // created here (destroyed here)
	bool userStream = false;  // set by pwa_isobar_set_stream: device-buffer calls are asynchronous
	~pwa_isobar()
	{
		if (ownStream && stream)
			cudaStreamDestroy(stream);
	}
};

namespace {

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// the plan's arrays in one device buffer; devView points into it
int uploadPlan(pwa_isobar* A)
{
	iso::Plan& p = A->plan;
	const std::string why =
	    iso::buildPlan(A->waves, A->masses, A->species, A->beamMass, A->reflBasis, A->bose, A->spaceInversion,
	                   A->reflection, A->canonical, A->isospinSym ? &A->isospin : nullptr, p);
	if (!why.empty())
		return setError(kErrArg, why);
	const size_t oWaves = 0;
	const size_t oOrder = align16(oWaves + p.waves.size() * sizeof(iso::WaveDev));
	const size_t oLams = align16(oOrder + p.order.size() * sizeof(int32_t));
	const size_t oTerms = align16(oLams + p.lams.size() * sizeof(iso::LamTerm));
	const size_t oPoly = align16(oTerms + p.dterms.size() * sizeof(iso::DTerm));
	const size_t oNorm = align16(oPoly + sizeof(p.bfPoly));
	const size_t oPolyF = align16(oNorm + sizeof(p.bfNorm));
	const size_t oNormF = align16(oPolyF + sizeof(p.bfPolyF));
	const size_t oPerms = align16(oNormF + sizeof(p.bfNormF));
	const size_t oTermsS = align16(oPerms + p.perms.size() * sizeof(int32_t));
	const size_t total = align16(oTermsS + p.terms.size() * sizeof(iso::SymTerm));
	std::vector<unsigned char> h(total, 0);
	auto put = [&](size_t off, const void* src, size_t bytes) {
		if (bytes)
			std::memcpy(h.data() + off, src, bytes);
	};
	put(oWaves, p.waves.data(), p.waves.size() * sizeof(iso::WaveDev));
	put(oOrder, p.order.data(), p.order.size() * sizeof(int32_t));
	put(oLams, p.lams.data(), p.lams.size() * sizeof(iso::LamTerm));
	put(oTerms, p.dterms.data(), p.dterms.size() * sizeof(iso::DTerm));
	put(oPoly, p.bfPoly, sizeof(p.bfPoly));
	put(oNorm, p.bfNorm, sizeof(p.bfNorm));
	put(oPolyF, p.bfPolyF, sizeof(p.bfPolyF));
	put(oNormF, p.bfNormF, sizeof(p.bfNormF));
	put(oPerms, p.perms.data(), p.perms.size() * sizeof(int32_t));
	put(oTermsS, p.terms.data(), p.terms.size() * sizeof(iso::SymTerm));
	PWA_TRY(A->dPlan.ensure(total, "isobar wave plan"));
	PWA_TRY(cudaCheck(cudaMemcpyAsync(A->dPlan.p, h.data(), total, cudaMemcpyHostToDevice, A->stream), "plan upload"));
	PWA_TRY(cudaCheck(cudaStreamSynchronize(A->stream), "plan upload"));
	unsigned char* d = A->dPlan.as<unsigned char>();
	iso::PlanView v = p.view();
	v.waves = reinterpret_cast<const iso::WaveDev*>(d + oWaves);
	v.order = reinterpret_cast<const int32_t*>(d + oOrder);
	v.lams = reinterpret_cast<const iso::LamTerm*>(d + oLams);
	v.dterms = reinterpret_cast<const iso::DTerm*>(d + oTerms);
	v.bfPoly = reinterpret_cast<const double*>(d + oPoly);
	v.bfNorm = reinterpret_cast<const double*>(d + oNorm);
	v.bfPolyF = reinterpret_cast<const float*>(d + oPolyF);
	v.bfNormF = reinterpret_cast<const float*>(d + oNormF);
	v.perms = reinterpret_cast<const int32_t*>(d + oPerms);
	v.terms = reinterpret_cast<const iso::SymTerm*>(d + oTermsS);
	A->devView = v;
	A->dirty = false;
	return kOk;
}

}  // namespace

extern "C" {

int pwa_isobar_create(pwa_isobar** out)
{
	if (!out)
		return setError(kErrArg, "null argument");
	*out = new (std::nothrow) pwa_isobar();
	return *out ? kOk : setError(kErrOom, "out of host memory");
}

int pwa_isobar_destroy(pwa_isobar* A)
{
	delete A;
	return kOk;
}

int pwa_isobar_set_final_state(pwa_isobar* A, uint32_t nFs, const double* masses, const int32_t* species,
                               double beamMass)
{
	if (!A || !masses || !species)
		return setError(kErrArg, "null argument");
	if (nFs != 3)
		return setError(kErrUnsupported, "the isobar amplitudes cover three final-state particles");
	for (int i = 0; i < 3; ++i)
		if (!(masses[i] > 0.0) || !std::isfinite(masses[i]))
			return setError(kErrArg, "final-state masses must be positive");
	if (!(beamMass >= 0.0) || !std::isfinite(beamMass))
		return setError(kErrArg, "the beam mass must be >= 0");
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			if (species[i] == species[j] && masses[i] != masses[j])
				return setError(kErrArg, "identical particles must have equal masses");
	for (int i = 0; i < 3; ++i) {
		A->masses[i] = masses[i];
		A->species[i] = species[i];
	}
	A->beamMass = beamMass;
	A->finalState = true;
	A->dirty = true;
	return kOk;
}

int pwa_isobar_set_stream(pwa_isobar* A, void* s)
{
	if (!A)
		return setError(kErrArg, "null argument");
	if (A->ownStream && A->stream) {
		cudaStreamSynchronize(A->stream);
		cudaStreamDestroy(A->stream);
	}
	A->ownStream = false;
	A->userStream = true;
	A->stream = static_cast<cudaStream_t>(s);  // NULL: the CUDA default stream
	return kOk;
}

int pwa_isobar_set_formalism(pwa_isobar* A, int formalism)
{
	if (!A)
		return setError(kErrArg, "null argument");
	if (formalism != PWA_FORMALISM_HELICITY && formalism != PWA_FORMALISM_CANONICAL)
		return setError(kErrArg, "formalism must be PWA_FORMALISM_HELICITY or PWA_FORMALISM_CANONICAL");
	A->canonical = formalism == PWA_FORMALISM_CANONICAL;
	A->dirty = true;
	return kOk;
}

int pwa_isobar_set_chunk_events(pwa_isobar* A, uint64_t events)
{
	if (!A)
		return setError(kErrArg, "null argument");
	A->chunkEvents = events;
	return kOk;
}

int pwa_isobar_set_options(pwa_isobar* A, int reflectivityBasis, int boseSymmetrize, int spaceInversion, int reflection)
{
	if (!A)
		return setError(kErrArg, "null argument");
	if (reflectivityBasis)
		for (const pwa_isobar_wave& w : A->waves)
			if (w.M < 0)
				return setError(kErrArg, "the reflectivity basis needs M >= 0 for every wave");
	A->reflBasis = reflectivityBasis != 0;
	A->bose = boseSymmetrize != 0;
	A->spaceInversion = spaceInversion != 0;
	A->reflection = reflection != 0;
	A->dirty = true;
	return kOk;
}

int pwa_isobar_add_wave(pwa_isobar* A, const pwa_isobar_wave* w)
{
	if (!A || !w)
		return setError(kErrArg, "null argument");
	const std::string why = iso::checkWave(*w, A->reflBasis);
	if (!why.empty())
		return setError(kErrArg, "pwa_isobar_add_wave: " + why);
	A->waves.push_back(*w);
	A->dirty = true;
	return kOk;
}

int pwa_isobar_nmb_waves(const pwa_isobar* A, uint32_t* n)
{
	if (!A || !n)
		return setError(kErrArg, "null argument");
	*n = (uint32_t)A->waves.size();
	return kOk;
}

int pwa_isobar_nmb_sym_terms(const pwa_isobar* A, uint32_t wave, uint32_t* n)
{
	if (!A || !n)
		return setError(kErrArg, "null argument");
	if (wave >= A->waves.size())
		return setError(kErrArg, "wave index out of range");
	if (A->isospinSym && !A->isospinSet)
		return setError(kErrState, "isospin symmetrisation needs the final-state isospins");
	*n = (uint32_t)iso::symTerms(A->waves[wave], A->species, A->bose, A->isospinSym ? &A->isospin : nullptr).size();
	return kOk;
}

int pwa_isobar_set_isospins(pwa_isobar* A, const int32_t* I, const int32_t* I3, const int32_t* P)
{
	if (!A || !I || !I3 || !P)
		return setError(kErrArg, "null argument");
	for (int i = 0; i < 3; ++i)
		if (I[i] < 0 || std::abs(I3[i]) > I[i] || ((I[i] - I3[i]) & 1) || (P[i] != 1 && P[i] != -1))
			return setError(kErrArg, "isospins need 0 <= |2I_3| <= 2I of equal parity and parities +-1");
	for (int i = 0; i < 3; ++i) {
		A->isospin.I[i] = I[i];
		A->isospin.I3[i] = I3[i];
		A->isospin.P[i] = P[i];
	}
	A->isospinSet = true;
	A->dirty = true;
	return kOk;
}

int pwa_isobar_enable_isospin_symmetrization(pwa_isobar* A, int flag)
{
	if (!A)
		return setError(kErrArg, "null argument");
	if (flag && !A->isospinSet)
		return setError(kErrState, "set the final-state isospins first");
	A->isospinSym = flag != 0;
	A->dirty = true;
	return kOk;
}

int pwa_isobar_amplitudes(pwa_isobar* A, const double* beam, const double* fs, uint64_t n, void* amps, int ampType,
                          int memory)
{
	if (!A)
		return setError(kErrArg, "null argument");
	if (ampType != PWA_COMPLEX64 && ampType != PWA_COMPLEX128)
		return setError(kErrArg, "ampType must be PWA_COMPLEX64 or PWA_COMPLEX128");
	const bool fp32 = ampType == PWA_COMPLEX64;
	const uint64_t ampBytes = fp32 ? 8 : 16;
	if (memory != PWA_MEMORY_HOST && memory != PWA_MEMORY_DEVICE)
		return setError(kErrArg, "memory must be PWA_MEMORY_HOST or PWA_MEMORY_DEVICE");
	if (!A->finalState)
		return setError(kErrState, "set the final state first");
	if (A->waves.empty())
		return setError(kErrState, "no waves");
	if (n == 0)
		return kOk;
	if (!beam || !fs || !amps)
		return setError(kErrArg, "null buffer");
	const uint64_t W = A->waves.size();
	if (n > (uint64_t)1 << 40 || W * n > ((uint64_t)1 << 62) / ampBytes)
		return setError(kErrArg, "too many events");
	if (!A->stream && !A->userStream) {
		PWA_TRY(cudaCheck(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking), "stream create"));
		A->ownStream = true;
	}
	if (A->dirty)
		PWA_TRY(uploadPlan(A));
	if (memory == PWA_MEMORY_HOST) {
		// slabs of events: rows [3][slab] and [9][slab] taken from the host's
		// [3][n] and [9][n], amplitude rows [W][slab] put back into [W][n], so
		// the device buffers stay bounded
		const uint64_t perEvent = 12 * sizeof(double) + W * ampBytes;
		const uint64_t slab = std::min<uint64_t>(n, A->chunkEvents ? A->chunkEvents
		                                                              : std::max<uint64_t>(1, (1ull << 30) / perEvent));
		PWA_TRY(A->dIn.ensure(slab * 12 * sizeof(double), "isobar event buffer"));
		PWA_TRY(A->dOut.ensure(W * slab * ampBytes, "isobar amplitude buffer"));
		double* in = A->dIn.as<double>();
		// one copy per row (no pitch limit for long rows)
		for (uint64_t e0 = 0; e0 < n; e0 += slab) {
			const uint64_t m = std::min(slab, n - e0);
			for (uint64_t r = 0; r < 12; ++r) {
				const double* src = (r < 3 ? beam + r * n : fs + (r - 3) * n) + e0;
				PWA_TRY(cudaCheck(cudaMemcpyAsync(in + r * m, src, m * sizeof(double), cudaMemcpyHostToDevice,
				                                  A->stream),
				                  "momentum upload"));
			}
			PWA_TRY(launchIsobarAmplitudes(A->devView, in, in + 3 * m, m, A->dOut.p, fp32, A->stream));
			for (uint64_t w = 0; w < W; ++w)
				PWA_TRY(cudaCheck(cudaMemcpyAsync(static_cast<unsigned char*>(amps) + (w * n + e0) * ampBytes,
				                                  static_cast<const unsigned char*>(A->dOut.p) + w * m * ampBytes,
				                                  m * ampBytes, cudaMemcpyDeviceToHost, A->stream),
				                  "amplitude download"));
		}
		return cudaCheck(cudaStreamSynchronize(A->stream), "isobar amplitudes");
	}
	if (!A->userStream)
		PWA_TRY(cudaCheck(cudaDeviceSynchronize(), "synchronise before reading device momenta"));
	PWA_TRY(launchIsobarAmplitudes(A->devView, beam, fs, n, amps, fp32, A->stream));
	// on the caller's stream, device-buffer calls stay asynchronous (stream order)
	if (A->userStream)
		return kOk;
	return cudaCheck(cudaStreamSynchronize(A->stream), "isobar amplitudes");
}

// calcAmplitudes (pyInterface/scripts/calcAmplitudes.py, which writes one
// amplitude tree per wave): the amplitudes of every wave for host momenta,
// computed in slabs and written as complex64 rows of one raw amplitude file,
// with the final-state mass ("mass") and the caller's variables as binning
// variables
int pwa_isobar_write_amp_file(pwa_isobar* A, const char* path, const char* const* waveNames, const double* beam,
                              const double* fs, uint64_t n, uint32_t nVars, const char* const* varNames,
                              const double* vars)
{
	if (!A || !path || !waveNames || (n && (!beam || !fs)) || (nVars && (!varNames || !vars)))
		return setError(kErrArg, "null argument");
	if (!A->finalState)
		return setError(kErrState, "set the final state first");
	const uint32_t W = (uint32_t)A->waves.size();
	if (W == 0)
		return setError(kErrState, "no waves");
	std::vector<const char*> names(waveNames, waveNames + W);
	names.push_back("mass");
	for (uint32_t v = 0; v < nVars; ++v) {
		if (varNames[v] && std::strcmp(varNames[v], "mass") == 0)
			return setError(kErrArg, "binning variable 'mass' is written by the call itself (the final-state mass)");
		names.push_back(varNames[v]);
	}
	std::vector<unsigned char> header;
	PWA_TRY(ampFileHeader(W, nVars + 1, names.data(), n, header));
	const uint64_t data = header.size();
	// written to <path>.tmp and renamed at the end: an error part-way leaves
	// no file behind
	AmpFileWriter out;
	PWA_TRY(out.create(path));
	const int fd = out.fd;
	PWA_TRY(ampFilePwrite(fd, header.data(), header.size(), 0, path));
	const uint64_t slab = std::min<uint64_t>(std::max<uint64_t>(n, 1), A->chunkEvents ? A->chunkEvents : 1u << 20);
	std::vector<double> b(3 * slab), f(9 * slab), mass(slab);
	std::vector<float> amps(2 * (size_t)W * slab);
	for (uint64_t e0 = 0; e0 < n; e0 += slab) {
		const uint64_t m = std::min(slab, n - e0);
		for (int r = 0; r < 3; ++r)
			std::copy(beam + r * n + e0, beam + r * n + e0 + m, b.begin() + r * m);
		for (int r = 0; r < 9; ++r)
			std::copy(fs + r * n + e0, fs + r * n + e0 + m, f.begin() + r * m);
		PWA_TRY(pwa_isobar_amplitudes(A, b.data(), f.data(), m, amps.data(), PWA_COMPLEX64, PWA_MEMORY_HOST));
		for (uint32_t w = 0; w < W; ++w)
			PWA_TRY(ampFilePwrite(fd, amps.data() + 2 * (size_t)w * m, m * 8, data + ((uint64_t)w * n + e0) * 8, path));
		// final-state mass from the momenta and the particle masses
		for (uint64_t e = 0; e < m; ++e) {
			double E = 0, px = 0, py = 0, pz = 0;
			for (int i = 0; i < 3; ++i) {
				const double x = f[(3 * i) * m + e], y = f[(3 * i + 1) * m + e], z = f[(3 * i + 2) * m + e];
				E += std::sqrt(A->masses[i] * A->masses[i] + (x * x + y * y + z * z));
				px += x;
				py += y;
				pz += z;
			}
			mass[e] = std::sqrt(std::max(0.0, E * E - (px * px + py * py + pz * pz)));
		}
		PWA_TRY(ampFilePwrite(fd, mass.data(), m * 8, data + (uint64_t)W * n * 8 + e0 * 8, path));
	}
	for (uint32_t v = 0; v < nVars; ++v)
		PWA_TRY(ampFilePwrite(fd, vars + (uint64_t)v * n, n * 8, data + ((uint64_t)W + 1 + v) * n * 8, path));
	return out.commit();
}

int pwa_clebsch_gordan(int32_t j1, int32_t m1, int32_t j2, int32_t m2, int32_t J, int32_t M, double* out)
{
	if (!out)
		return setError(kErrArg, "null argument");
	if (j1 > 2 * iso::kMaxSpin || j2 > 2 * iso::kMaxSpin || J > 4 * iso::kMaxSpin)
		return setError(kErrArg, "spins out of range");
	*out = iso::clebschGordan(j1, m1, j2, m2, J, M);
	return kOk;
}

int pwa_wigner_d(int32_t j, int32_t m, int32_t n, double theta, double* out)
{
	if (!out)
		return setError(kErrArg, "null argument");
	if (j < 0 || j > 2 * iso::kMaxSpin || std::abs(m) > j || std::abs(n) > j || ((j - m) & 1) || ((j - n) & 1))
		return setError(kErrArg, "illegal arguments of the Wigner d function");
	*out = iso::wignerD(j, m, n, theta);
	return kOk;
}

int pwa_barrier_factor(int32_t L, double q, double* out)
{
	if (!out)
		return setError(kErrArg, "null argument");
	if (L < 0 || L > iso::kMaxL || (L & 1))
		return setError(kErrArg, "2L must be even and in 0 .. 14");
	if (!(q >= 0.0))
		return setError(kErrArg, "q must be >= 0");
	double poly[8][8], norm[8];
	iso::barrierPolynomials(poly, norm);
	iso::PlanView v{};
	v.bfPoly = &poly[0][0];
	v.bfNorm = norm;
	*out = std::sqrt(iso::barrierF2(v, L, q));
	return kOk;
}

}  // extern "C"
