// C-ABI driver over the reference's own rpwa::pwaLikelihood and
// rpwa::ampIntegralMatrix -- TEST INFRASTRUCTURE ONLY.
//
// Built by `make -C oracle ref` together with the reference's unmodified
// sources partialWaveFit/pwaLikelihood.cc and
// decayAmplitude/ampIntegralMatrix.cc (compiled where they lie, through a
// directory of symlinks under oracle/_ref/src) against the shims in
// oracle/ref_shim (Boost containers and accumulator framework, ROOT
// stand-ins, in-memory amplitude and event trees).  The likelihood,
// gradient, Hessian, parameter layout, normalisation, integral and Kahan
// arithmetic that run are the reference's.  The tests use this library to
// pin the restated oracle (pwa_oracle.cpp) and to write golden fixtures; the
// product never loads it.
//
// The entry points take the same arguments as the oracle's (oracle_* ->
// ref_*), so one Python wrapper class serves both.
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <unistd.h>
#include <vector>

#include "ampIntegralMatrix.h"
#include "amplitudeMetadata.h"
#include "complexMatrix.h"
#include "eventMetadata.h"
#include "pwaLikelihood.h"

using namespace rpwa;
typedef std::complex<double>  cplx;
typedef pwaLikelihood<cplx>   Lik;

namespace {

	// the reference reports progress on std::cout; the tests want it quiet
	struct QuietCout {
		std::ostringstream sink;
		std::streambuf*    saved;
		QuietCout() : saved(std::cout.rdbuf(sink.rdbuf())) {}
		~QuietCout() { std::cout.rdbuf(saved); }
	};

	// one in-memory amplitude tree per wave
	struct WaveTree {
		std::unique_ptr<TTree>             tree;
		std::unique_ptr<amplitudeMetadata> meta;
	};

	WaveTree makeWaveTree(const std::string& name, const cplx* amps, unsigned long nEv, unsigned nSub,
	                      const std::vector<eventMetadata>& evtMetas)
	{
		WaveTree t;
		t.tree.reset(new TTree((long)nEv));
		t.tree->setAmplitudes(amps, nSub);
		t.meta.reset(new amplitudeMetadata(name, t.tree.get(), evtMetas));
		return t;
	}

	struct RefIntegral {
		ampIntegralMatrix m;
	};

	struct RefLikelihood {
		Lik                                  L;
		std::vector<eventMetadata>           evtMetas;   // on-the-fly binning: the one event file
		std::unique_ptr<TTree>               evtTree;
		std::vector<std::vector<double> >    binCols;
		unsigned long                        otfSelected = 0;
	};

	const cplx* asCplx(const double* p) { return reinterpret_cast<const cplx*>(p); }

}  // namespace


extern "C" {

// ---------------------------------------------------------------- integrals
void* ref_int_create() { return new RefIntegral(); }
void  ref_int_destroy(void* h) { delete (RefIntegral*)h; }

// ampIntegralMatrix::integrate over amplitude trees [wave][event][sub];
// weights (importance-sampling weights w, the reference uses 1/w) go through
// a temporary weight file as the reference reads them; inBin != null selects
// events through an on-the-fly bin on an event-tree column
int ref_int_integrate(void* h, unsigned nWaves, const char* const* names, const double* amps, unsigned long nEv,
                      unsigned nSub, const double* weights, unsigned long nWeights, const unsigned char* inBin,
                      long maxNmbEvents)
{
	QuietCout q;
	RefIntegral&           I = *(RefIntegral*)h;
	std::vector<WaveTree>  trees;
	std::vector<const amplitudeMetadata*> metas;
	for (unsigned w = 0; w < nWaves; ++w) {
		trees.push_back(makeWaveTree(names[w], asCplx(amps) + (size_t)w * nEv * nSub, nEv, nSub,
		                             std::vector<eventMetadata>()));
		metas.push_back(trees.back().meta.get());
	}
	std::string weightFile;
	if (weights) {
		char tmpl[] = "/tmp/pwa_ref_weightsXXXXXX";
		const int fd = mkstemp(tmpl);
		if (fd < 0)
			return 0;
		close(fd);
		weightFile = tmpl;
		std::ofstream out(weightFile);
		out.precision(17);
		for (unsigned long k = 0; k < nWeights; ++k)
			out << weights[k] << "\n";
	}
	std::unique_ptr<TTree>         evtTree;
	std::unique_ptr<eventMetadata> evtMeta;
	std::vector<double>            inBinCol;
	multibinBoundariesType         otfBin;
	if (inBin) {
		inBinCol.resize(nEv);
		for (unsigned long e = 0; e < nEv; ++e)
			inBinCol[e] = inBin[e] ? 1 : 0;
		evtTree.reset(new TTree((long)nEv));
		evtTree->addColumn("inBin", inBinCol.data());
		evtMeta.reset(new eventMetadata("mc", evtTree.get(), std::vector<std::string>(1, "inBin")));
		otfBin["inBin"] = boundaryType(0.5, 1.5);
	}
	bool ok;
	try {
		ok = I.m.integrate(metas, maxNmbEvents, weightFile, evtMeta.get(), otfBin);
	} catch (...) {
		ok = false;
	}
	if (!weightFile.empty())
		unlink(weightFile.c_str());
	return ok ? 1 : 0;
}

int ref_int_add_event(void* h, const double* amps)
{
	RefIntegral& I = *(RefIntegral*)h;
	std::map<std::string, cplx> a;
	for (unsigned i = 0; i < I.m.nmbWaves(); ++i)
		a[I.m.waveName(i)] = asCplx(amps)[i];
	return I.m.addEvent(a) ? 1 : 0;
}

int ref_int_set_wave_names(void* h, unsigned n, const char* const* names)
{
	QuietCout q;
	std::vector<std::string> v(names, names + n);
	return ((RefIntegral*)h)->m.setWaveNames(v) ? 1 : 0;
}

void ref_int_element(void* h, unsigned i, unsigned j, double* out)
{
	const cplx c = ((RefIntegral*)h)->m.element(i, j);
	out[0] = c.real();
	out[1] = c.imag();
}

void ref_int_raw(void* h, double* out)
{
	const ampIntegralMatrix& m = ((RefIntegral*)h)->m;
	for (unsigned i = 0; i < m.nmbWaves(); ++i)
		for (unsigned j = 0; j < m.nmbWaves(); ++j) {
			const cplx c = m.matrix()[i][j];
			out[2 * ((size_t)i * m.nmbWaves() + j)]     = c.real();
			out[2 * ((size_t)i * m.nmbWaves() + j) + 1] = c.imag();
		}
}

void ref_int_set_raw(void* h, const double* in)
{
	ampIntegralMatrix& m = ((RefIntegral*)h)->m;
	for (unsigned i = 0; i < m.nmbWaves(); ++i)
		for (unsigned j = 0; j < m.nmbWaves(); ++j)
			m.matrix()[i][j] = asCplx(in)[(size_t)i * m.nmbWaves() + j];
}

unsigned long ref_int_nmb_events(void* h) { return ((RefIntegral*)h)->m.nmbEvents(); }
void          ref_int_set_nmb_events(void* h, unsigned long n) { ((RefIntegral*)h)->m.setNmbEvents(n); }
unsigned      ref_int_nmb_waves(void* h) { return ((RefIntegral*)h)->m.nmbWaves(); }

int ref_int_add(void* h, void* o)
{
	QuietCout q;
	try {
		((RefIntegral*)h)->m += ((RefIntegral*)o)->m;
	} catch (...) {
		return 0;
	}
	return 1;
}

int ref_int_read_ascii(void* h, const char* path)
{
	QuietCout q;
	return ((RefIntegral*)h)->m.readAscii(std::string(path)) ? 1 : 0;
}

int ref_int_write_ascii(void* h, const char* path)
{
	QuietCout q;
	return ((RefIntegral*)h)->m.writeAscii(std::string(path)) ? 1 : 0;
}

int ref_int_wave_name(void* h, unsigned i, char* buf, unsigned len)
{
	const std::string& s = ((RefIntegral*)h)->m.waveName(i);
	std::snprintf(buf, len, "%s", s.c_str());
	return 1;
}

// --------------------------------------------------------------- likelihood
void* ref_lik_create()
{
	Lik::setQuiet(true);
	QuietCout q;
	return new RefLikelihood();
}
void ref_lik_destroy(void* h) { delete (RefLikelihood*)h; }

void ref_lik_set_options(void* h, int useNormalizedAmps, int prior, double cauchyWidth)
{
	Lik& L = ((RefLikelihood*)h)->L;
	L.useNormalizedAmps(useNormalizedAmps != 0);
	L.setPriorType(prior ? Lik::HALF_CAUCHY : Lik::FLAT);
	L.setCauchyWidth(cauchyWidth);
}

// pwaLikelihood::setOnTheFlyBinning over one event file whose binning
// variables are the given columns
int ref_lik_set_otf_binning(void* h, unsigned nVars, const double* lower, const double* upper,
                            const void* const* cols, unsigned long nEv, const char* const* names)
{
	QuietCout q;
	RefLikelihood& R = *(RefLikelihood*)h;
	R.evtTree.reset(new TTree((long)nEv));
	R.binCols.assign(nVars, std::vector<double>());
	multibinBoundariesType bounds;
	std::vector<std::string> varNames;
	for (unsigned v = 0; v < nVars; ++v) {
		const double* c = (const double*)cols[v];
		R.binCols[v].assign(c, c + nEv);
		R.evtTree->addColumn(names[v], R.binCols[v].data());
		bounds[names[v]] = boundaryType(lower[v], upper[v]);
		varNames.push_back(names[v]);
	}
	R.evtMetas.assign(1, eventMetadata("data", R.evtTree.get(), varNames));
	std::vector<const eventMetadata*> metas(1, &R.evtMetas[0]);
	if (not R.L.setOnTheFlyBinning(bounds, metas))
		return 0;
	// count the selected events the way addAmplitude will see them
	std::map<std::string, double> vals;
	unsigned long n = 0;
	for (unsigned long e = 0; e < nEv; ++e) {
		bool in = true;
		for (unsigned v = 0; v < nVars; ++v)
			if (R.binCols[v][e] < lower[v] or R.binCols[v][e] >= upper[v])
				in = false;
		n += in ? 1 : 0;
	}
	R.otfSelected = n;
	return 1;
}

unsigned long ref_lik_otf_selected(void* h) { return ((RefLikelihood*)h)->otfSelected; }

int ref_lik_init(void* h, unsigned nWaves, const char* const* names, const int* refl, const double* thresholds,
                 unsigned rank, double massBinCenter)
{
	QuietCout q;
	std::vector<Lik::waveDescThresType> waves;
	for (unsigned w = 0; w < nWaves; ++w)
		waves.push_back(Lik::waveDescThresType(names[w], waveDescription(refl[w] > 0 ? +1 : -1),
		                                       thresholds ? thresholds[w] : 0.));
	return ((RefLikelihood*)h)->L.init(waves, rank, massBinCenter) ? 1 : 0;
}

int ref_lik_add_norm_integral(void* h, void* integral)
{
	QuietCout q;
	return ((RefLikelihood*)h)->L.addNormIntegral(((RefIntegral*)integral)->m) ? 1 : 0;
}

int ref_lik_add_acc_integral(void* h, void* integral, unsigned long accEventsOverride)
{
	QuietCout q;
	return ((RefLikelihood*)h)->L.addAccIntegral(((RefIntegral*)integral)->m, (unsigned)accEventsOverride) ? 1 : 0;
}

int ref_lik_add_amplitude(void* h, const char* name, const double* amps, unsigned long nEv)
{
	QuietCout q;
	RefLikelihood& R = *(RefLikelihood*)h;
	WaveTree t = makeWaveTree(name, asCplx(amps), nEv, 1, R.evtMetas);
	std::vector<const amplitudeMetadata*> metas(1, t.meta.get());
	try {
		return R.L.addAmplitude(metas) ? 1 : 0;
	} catch (...) {
		return 0;
	}
}

int ref_lik_finish_init(void* h)
{
	QuietCout q;
	return ((RefLikelihood*)h)->L.finishInit() ? 1 : 0;
}

unsigned ref_lik_nmb_pars(void* h) { return ((RefLikelihood*)h)->L.nmbPars(); }
unsigned ref_lik_nmb_pars_fixed(void* h) { return ((RefLikelihood*)h)->L.nmbParsFixed(); }
int      ref_lik_par_fixed(void* h, unsigned i) { return ((RefLikelihood*)h)->L.parameter(i).fixed() ? 1 : 0; }
unsigned ref_lik_nmb_waves(void* h, int refl) { return ((RefLikelihood*)h)->L.nmbWaves(refl); }
unsigned ref_lik_nmb_events(void* h) { return ((RefLikelihood*)h)->L.nmbEvents(); }

int ref_lik_par_name(void* h, unsigned i, char* buf, unsigned len)
{
	std::snprintf(buf, len, "%s", ((RefLikelihood*)h)->L.parameter(i).parName().c_str());
	return 1;
}

void ref_lik_fdf(void* h, const double* par, double* f, double* grad, unsigned /*threads*/)
{
	QuietCout q;
	((RefLikelihood*)h)->L.FdF(par, *f, grad);
}

double ref_lik_doeval(void* h, const double* par, unsigned /*threads*/)
{
	QuietCout q;
	return ((RefLikelihood*)h)->L.DoEval(par);
}

void ref_lik_gradient(void* h, const double* par, double* grad, unsigned /*threads*/)
{
	QuietCout q;
	((RefLikelihood*)h)->L.Gradient(par, grad);
}

double ref_lik_doderivative(void* h, const double* par, unsigned i)
{
	QuietCout q;
	return ((RefLikelihood*)h)->L.DoDerivative(par, i);
}

double ref_lik_dlcache(void* h, unsigned i) { return ((RefLikelihood*)h)->L.dLcache(i); }

void ref_lik_hessian(void* h, const double* par, double* out)
{
	QuietCout q;
	const Lik&             L = ((RefLikelihood*)h)->L;
	const TMatrixT<double> H = L.Hessian(par);
	const unsigned         n = L.nmbPars();
	for (unsigned i = 0; i < n; ++i)
		for (unsigned j = 0; j < n; ++j)
			out[(size_t)i * n + j] = H[i][j];
}

int ref_lik_covariance(void* h, const double* hessian, double* out)
{
	QuietCout q;
	const Lik&       L = ((RefLikelihood*)h)->L;
	const unsigned   n = L.nmbPars();
	TMatrixT<double> H(n, n);
	for (unsigned i = 0; i < n; ++i)
		for (unsigned j = 0; j < n; ++j)
			H[i][j] = hessian[(size_t)i * n + j];
	try {
		const TMatrixT<double> C = L.CovarianceMatrix(H);
		for (unsigned i = 0; i < n; ++i)
			for (unsigned j = 0; j < n; ++j)
				out[(size_t)i * n + j] = C[i][j];
	} catch (...) {
		return 0;
	}
	return 1;
}

void ref_lik_correct_param_signs(void* h, const double* par, double* out)
{
	QuietCout q;
	const std::vector<double> v = ((RefLikelihood*)h)->L.CorrectParamSigns(par);
	std::copy(v.begin(), v.end(), out);
}

// getIntegralMatrices (normalisation, acceptance, phase-space integrals) in
// the likelihood's wave order
void ref_lik_integral_matrices(void* h, double* norm, double* acc, double* ps, int withFlat)
{
	QuietCout q;
	complexMatrix       N, A;
	std::vector<double> P;
	((RefLikelihood*)h)->L.getIntegralMatrices(N, A, P, withFlat != 0);
	for (unsigned i = 0; i < N.nRows(); ++i)
		for (unsigned j = 0; j < N.nCols(); ++j) {
			const size_t k = (size_t)i * N.nCols() + j;
			norm[2 * k]     = N.get(i, j).real();
			norm[2 * k + 1] = N.get(i, j).imag();
			acc[2 * k]      = A.get(i, j).real();
			acc[2 * k + 1]  = A.get(i, j).imag();
		}
	std::copy(P.begin(), P.end(), ps);
}

}  // extern "C"
