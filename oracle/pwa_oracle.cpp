// pwa_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// FP64 CPU restatement of the ROOTPWA extended-likelihood hot path, used as the
// checker for the CUDA product (tests, the smoke check and the CPU-baseline leg
// of bench.py).  Nothing in the product links, loads or calls this file.
//
// Parity status: pinned against the reference's own code.  `make ref` in this
// directory compiles the reference's pwaLikelihood.cc and ampIntegralMatrix.cc
// from their sources against local stand-ins for ROOT and Boost (ref_shim/),
// and tests/test_ref_pinned.py finds this restatement bit for bit equal to them
// (integrals, FdF / DoEval / Gradient, Hessian, parameter layout, on-the-fly
// binning).  Also pinned by the reference's ASCII integral fixture
// (test/decayAmplitude/testIntegral.int, read and re-written bit-exactly), by
// central finite differences and by the analytic identities of
// doc/tex/likelihood.tex.
//
// The summation semantics follow the reference exactly: event-major loops,
// a compensated (Kahan) accumulator at every summation level
// (utilities/sumAccumulators.hpp:152-192), complex<double> arithmetic, and a
// per-event heap temporary in FdF/Gradient (partialWaveFit/pwaLikelihood.cc:215)
// so that the single-thread CPU timing is representative of the reference.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

typedef std::complex<double> cplx;

// Compensated (Kahan) sum; one step per sample as in
// utilities/sumAccumulators.hpp:165-178.  For complex samples the real and
// imaginary parts are compensated independently, which is what the
// reference's template does since complex +/- act componentwise.
template <typename T>
struct kahan {
	T s = T();
	T c = T();
	void operator()(const T& x)
	{
		const T y = x - c;
		const T t = s + y;
		c = (t - s) - y;
		s = t;
	}
	T sum() const { return s; }
};

// Half-Cauchy prior helpers, partialWaveFit/pwaLikelihood.cc:78-102.
double cauchyF(double x, double g) { return 1. / (1. + (x * x) / (g * g)); }
double cauchyD(double x, double g) { return (-2. * x * g * g) / ((g * g + x * x) * (g * g + x * x)); }
double cauchyD2(double x, double g)
{
	const double x2 = x * x, g2 = g * g;
	return g2 / ((g2 + x2) * (g2 + x2)) * (-2. + 8. * x2 / (g2 + x2));
}

// ---------------------------------------------------------------------------
// ampIntegralMatrix restatement (decayAmplitude/ampIntegralMatrix.{h,cc})
// ---------------------------------------------------------------------------
struct OracleIntegral {
	unsigned int              nmbWaves = 0;
	unsigned long             nmbEvents = 0;
	std::vector<std::string>  waveNames;
	std::vector<cplx>         sums;  // raw sums, row-major [i][j]

	int waveIndex(const std::string& n) const
	{
		for (size_t i = 0; i < waveNames.size(); ++i)
			if (waveNames[i] == n)
				return (int)i;
		return -1;
	}
	// element = raw sum / nmbEvents (ampIntegralMatrix.cc:237-252)
	cplx element(unsigned i, unsigned j) const { return sums[(size_t)i * nmbWaves + j] / ((double)nmbEvents); }
};

// ---------------------------------------------------------------------------
// pwaLikelihood restatement (partialWaveFit/pwaLikelihood.{h,cc})
// ---------------------------------------------------------------------------
struct ParInfo {
	std::string waveName;
	int         rank;
	double      threshold;
	bool        fixed;
	bool        realPart;
};

struct OracleLikelihood {
	// options
	bool   useNormalizedAmps = true;   // pwaLikelihood.cc:147
	int    priorType = 0;              // 0 = FLAT, 1 = HALF_CAUCHY
	double cauchyWidth = 0.5;          // pwaLikelihood.cc:149
	// event shard: only the root shard adds normalisation and prior (the
	// product's pwa_likelihood_set_shard; no reference counterpart)
	bool   shardSet = false, shardRoot = true;
	unsigned long shardTotal = 0;
	double normFactor() const
	{
		if (shardSet && !shardRoot) return 0.;
		if (useNormalizedAmps) return 1.;
		return (double)(shardSet ? shardTotal : nEvents);
	}
	int effPrior() const { return (shardSet && !shardRoot) ? 0 : priorType; }
	// on-the-fly binning (pwaLikelihood.cc:1391-1440): file indices of the
	// events with lower <= x < upper for every binning variable
	bool otfSet = false;
	unsigned long otfFileEvents = 0;
	std::vector<unsigned long> otfIdx;
	bool setOtf(unsigned nVars, const double* lower, const double* upper, const double* const* vars,
	            unsigned long nFile)
	{
		if (nEvents != 0 or nFile == 0)
			return false;
		otfSet = true;
		otfFileEvents = nFile;
		otfIdx.clear();
		for (unsigned long i = 0; i < nFile; ++i) {
			bool use = true;
			for (unsigned v = 0; v < nVars; ++v)
				if (vars[v][i] < lower[v] or vars[v][i] >= upper[v])
					use = false;
			if (use)
				otfIdx.push_back(i);
		}
		return true;
	}

	// wave set
	unsigned int nW[2] = {0, 0};       // [0] = negative, [1] = positive reflectivity
	unsigned int nWmax = 0;
	unsigned int rank = 1;
	std::vector<std::string> waveNames[2];
	std::vector<double>      waveThres[2];
	std::map<std::string, std::pair<unsigned, unsigned> > waveParams;  // name -> (refl, index)

	// parameter layout (pwaLikelihood.cc:1487-1556)
	unsigned int nPars = 0, nParsFixed = 0;
	std::vector<ParInfo> pars;
	std::vector<int> mapRe, mapIm;     // [rank][2][nWmax] -> parameter index or -1

	// integrals, reordered [refl][i][refl][j] (pwaLikelihood.cc:1559-1574)
	std::vector<cplx> normM, accM;
	unsigned long numbAccEvents = 0;
	double totAcc = 0;
	std::vector<double> phaseSpaceIntegral;

	// decay amplitudes [refl][event][wave] (pwaLikelihood.h:309)
	unsigned long nEvents = 0;
	std::vector<cplx> amps[2];
	std::vector<char> ampAdded[2];

	bool initialized = false, normAdded = false, accAdded = false, finished = false;

	size_t pIdx(unsigned r, unsigned e, unsigned w) const { return ((size_t)r * 2 + e) * nWmax + w; }
	size_t mIdx(unsigned e1, unsigned i, unsigned e2, unsigned j) const
	{
		return (((size_t)e1 * nWmax + i) * 2 + e2) * nWmax + j;
	}

	// pwaLikelihood.cc:1443-1556
	bool init(unsigned n, const char* const* names, const int* refl, const double* thres, unsigned rk,
	          double massBinCenter)
	{
		for (unsigned i = 0; i < n; ++i) {
			const unsigned e = (refl[i] > 0) ? 1 : 0;
			++nW[e];
			waveNames[e].push_back(names[i]);
			waveThres[e].push_back(thres ? thres[i] : 0.);
		}
		nWmax = std::max(nW[0], nW[1]);
		for (unsigned e = 0; e < 2; ++e) {
			ampAdded[e].assign(nWmax, 0);
			for (unsigned w = 0; w < nW[e]; ++w)
				waveParams[waveNames[e][w]] = std::make_pair(e, w);
		}
		if (nW[0] + nW[1] == 0)
			return false;
		rank = rk;
		nPars = 0;
		for (unsigned r = 0; r < rank; ++r) {
			const int pos = (int)nW[1] - (int)r, neg = (int)nW[0] - (int)r;
			const int posC = std::max(pos - 1, 0), negC = std::max(neg - 1, 0);
			nPars += 2 * (posC + negC);
			if (pos > 0) ++nPars;
			if (neg > 0) ++nPars;
		}
		nPars += 1;
		nParsFixed = 0;
		pars.assign(nPars, ParInfo());
		mapRe.assign((size_t)rank * 2 * nWmax, -1);
		mapIm.assign((size_t)rank * 2 * nWmax, -1);
		unsigned p = 0;
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned w = 0; w < nW[e]; ++w) {
					const double th = waveThres[e][w];
					const bool fixed = (th != 0 and th >= massBinCenter);
					if (w < r)
						continue;
					if (w == r) {
						pars[p] = ParInfo{waveNames[e][w], (int)r, th, fixed, true};
						if (fixed) ++nParsFixed;
						mapRe[pIdx(r, e, w)] = p;
						++p;
					} else {
						pars[p] = ParInfo{waveNames[e][w], (int)r, th, fixed, true};
						pars[p + 1] = ParInfo{waveNames[e][w], (int)r, th, fixed, false};
						if (fixed) nParsFixed += 2;
						mapRe[pIdx(r, e, w)] = p;
						mapIm[pIdx(r, e, w)] = p + 1;
						p += 2;
					}
				}
		pars[p] = ParInfo{"flat", 0, 0., false, true};
		initialized = true;
		return true;
	}

	// pwaLikelihood.cc:1559-1574: only same-reflectivity blocks are filled
	bool reorder(const OracleIntegral& I, std::vector<cplx>& out) const
	{
		out.assign((size_t)2 * nWmax * 2 * nWmax, cplx(0, 0));
		for (unsigned e = 0; e < 2; ++e)
			for (unsigned i = 0; i < nW[e]; ++i)
				for (unsigned j = 0; j < nW[e]; ++j) {
					const int a = I.waveIndex(waveNames[e][i]), b = I.waveIndex(waveNames[e][j]);
					if (a < 0 or b < 0)
						return false;
					out[mIdx(e, i, e, j)] = I.element(a, b);
				}
		return true;
	}

	// pwaLikelihood.cc:1066-1083
	bool addNormIntegral(const OracleIntegral& I)
	{
		if (not initialized)
			return false;
		numbAccEvents = I.nmbEvents;
		if (not reorder(I, normM))
			return false;
		normAdded = true;
		return true;
	}

	// pwaLikelihood.cc:1086-1107 (the argument's event count is overwritten, as in the reference)
	bool addAccIntegral(OracleIntegral& I, unsigned long override_)
	{
		if (not normAdded)
			return false;
		numbAccEvents = (override_ == 0) ? numbAccEvents : override_;
		totAcc = (double)I.nmbEvents / numbAccEvents;
		I.nmbEvents = numbAccEvents;
		if (not reorder(I, accM))
			return false;
		accAdded = true;
		return true;
	}

	// pwaLikelihood.cc:1110-1288 without the ROOT tree I/O: one wave's amplitudes
	// for all events arrive as an array.
	bool addAmplitude(const char* name, const double* a, unsigned long n)
	{
		if (not accAdded or n == 0)
			return false;
		std::vector<double> sel;
		if (otfSet) {
			if (n != otfFileEvents or otfIdx.empty())
				return false;
			sel.resize(2 * otfIdx.size());
			for (size_t k = 0; k < otfIdx.size(); ++k) {
				sel[2 * k] = a[2 * otfIdx[k]];
				sel[2 * k + 1] = a[2 * otfIdx[k] + 1];
			}
			a = sel.data();
			n = otfIdx.size();
		}
		auto it = waveParams.find(name);
		if (it == waveParams.end())
			return false;
		if (nEvents == 0) {
			nEvents = n;
			amps[0].assign((size_t)nEvents * nW[0], cplx(0, 0));
			amps[1].assign((size_t)nEvents * nW[1], cplx(0, 0));
		}
		if (n != nEvents)
			return false;
		const unsigned e = it->second.first, w = it->second.second;
		const cplx normInt = normM[mIdx(e, w, e, w)];
		bool fixPar = (accM[mIdx(e, w, e, w)] == 0.);
		for (unsigned long i = 0; i < nEvents; ++i) {
			cplx v(a[2 * i], a[2 * i + 1]);
			if (useNormalizedAmps) {
				if (normInt == 0. and v != 0.)
					return false;
				if (normInt != 0.)
					v /= std::sqrt(normInt.real());
			}
			if (v != 0.)
				fixPar = false;
			amps[e][i * nW[e] + w] = v;
		}
		if (fixPar)
			for (auto& p : pars)
				if (p.waveName == name and not p.fixed)
					p.fixed = true;
		ampAdded[e][w] = 1;
		return true;
	}

	// pwaLikelihood.cc:1291-1388
	bool finishInit()
	{
		for (unsigned e = 0; e < 2; ++e)
			for (unsigned w = 0; w < nW[e]; ++w)
				if (not ampAdded[e][w])
					return false;
		phaseSpaceIntegral.assign((size_t)2 * nWmax, 0.);
		for (unsigned e = 0; e < 2; ++e)
			for (unsigned w = 0; w < nW[e]; ++w)
				phaseSpaceIntegral[e * nWmax + w] = std::sqrt(normM[mIdx(e, w, e, w)].real());
		if (useNormalizedAmps) {
			for (unsigned e1 = 0; e1 < 2; ++e1)
				for (unsigned i = 0; i < nW[e1]; ++i) {
					double ni = std::sqrt(normM[mIdx(e1, i, e1, i)].real());
					if (ni == 0) ni = 1;
					for (unsigned e2 = 0; e2 < 2; ++e2)
						for (unsigned j = 0; j < nW[e2]; ++j) {
							double nj = std::sqrt(normM[mIdx(e2, j, e2, j)].real());
							if (nj == 0) nj = 1;
							if (e1 != e2 or i != j)
								normM[mIdx(e1, i, e2, j)] /= ni * nj;
							accM[mIdx(e1, i, e2, j)] /= ni * nj;
						}
				}
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned w = 0; w < nW[e]; ++w)
					if (normM[mIdx(e, w, e, w)] != 0.)
						normM[mIdx(e, w, e, w)] = 1;
		}
		finished = true;
		return true;
	}

	// pwaLikelihood.cc:1680-1708
	void fromPar(const double* par, std::vector<cplx>& V, double& flat) const
	{
		V.assign((size_t)rank * 2 * nWmax, cplx(0, 0));
		unsigned p = 0;
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned w = 0; w < nW[e]; ++w) {
					double re, im;
					if (w < r) {
						re = im = 0;
					} else if (w == r) {
						re = par[p];
						im = 0;
						++p;
					} else {
						re = par[p];
						im = par[p + 1];
						p += 2;
					}
					V[pIdx(r, e, w)] = cplx(re, im);
				}
		flat = par[p];
	}

	// pwaLikelihood.cc:1714-1731
	void toPar(const std::vector<cplx>& D, double flat, double* out) const
	{
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned w = 0; w < nW[e]; ++w) {
					const size_t k = pIdx(r, e, w);
					if (mapRe[k] >= 0) out[mapRe[k]] = D[k].real();
					if (mapIm[k] >= 0) out[mapIm[k]] = D[k].imag();
				}
		out[nPars - 1] = flat;
	}

	// Event-term of FdF / Gradient over events [b, e): pwaLikelihood.cc:209-244
	// (and :547-577).  withGrad=false gives the DoEval loop (:361-375).
	void eventLoop(const std::vector<cplx>& V, double flat, unsigned long b, unsigned long eEnd, bool withGrad,
	               kahan<double>& llAcc, std::vector<kahan<cplx> >& dAcc, kahan<double>& flatAcc) const
	{
		const double flat2 = flat * flat;
		const size_t nSlot = (size_t)rank * 2 * nWmax;
		for (unsigned long i = b; i < eEnd; ++i) {
			kahan<double> lAcc;
			// per-event heap temporary, as in pwaLikelihood.cc:215
			std::vector<cplx> deriv(withGrad ? nSlot : 0);
			for (unsigned r = 0; r < rank; ++r) {
				for (unsigned e = 0; e < 2; ++e) {
					kahan<cplx> sAcc;
					const cplx* A = &amps[e][(size_t)i * nW[e]];
					for (unsigned w = 0; w < nW[e]; ++w)
						sAcc(V[pIdx(r, e, w)] * A[w]);
					const cplx S = sAcc.sum();
					lAcc(std::norm(S));
					if (withGrad)
						for (unsigned w = 0; w < nW[e]; ++w)
							deriv[pIdx(r, e, w)] = S;
				}
				if (withGrad)
					for (unsigned e = 0; e < 2; ++e) {
						const cplx* A = &amps[e][(size_t)i * nW[e]];
						for (unsigned w = 0; w < nW[e]; ++w)
							deriv[pIdx(r, e, w)] *= std::conj(A[w]);
					}
			}
			lAcc(flat2);
			llAcc(-std::log(lAcc.sum()));
			if (withGrad) {
				const double factor = 2. / lAcc.sum();
				for (unsigned r = 0; r < rank; ++r)
					for (unsigned e = 0; e < 2; ++e)
						for (unsigned w = 0; w < nW[e]; ++w)
							dAcc[pIdx(r, e, w)](-factor * deriv[pIdx(r, e, w)]);
				flatAcc(-factor * flat);
			}
		}
	}

	// Full FdF (pwaLikelihood.cc:170-315).  nThreads > 1 splits the event loop
	// into contiguous chunks with their own accumulators (a parallelised
	// restatement, not reference behaviour), combined in chunk order.
	void fdf(const double* par, double* fOut, double* grad, bool withGrad, unsigned nThreads) const
	{
		std::vector<cplx> V;
		double flat;
		fromPar(par, V, flat);
		const double flat2 = flat * flat;
		const size_t nSlot = (size_t)rank * 2 * nWmax;
		kahan<double> llAcc, flatAcc;
		std::vector<kahan<cplx> > dAcc(nSlot);
		if (nThreads <= 1) {
			eventLoop(V, flat, 0, nEvents, withGrad, llAcc, dAcc, flatAcc);
		} else {
			std::vector<kahan<double> > ll(nThreads), fl(nThreads);
			std::vector<std::vector<kahan<cplx> > > d(nThreads, std::vector<kahan<cplx> >(nSlot));
			std::vector<std::thread> th;
			for (unsigned t = 0; t < nThreads; ++t) {
				const unsigned long b = nEvents * t / nThreads, e = nEvents * (t + 1) / nThreads;
				th.emplace_back([&, t, b, e]() { eventLoop(V, flat, b, e, withGrad, ll[t], d[t], fl[t]); });
			}
			for (auto& x : th) x.join();
			for (unsigned t = 0; t < nThreads; ++t) {
				llAcc(ll[t].sum());
				flatAcc(fl[t].sum());
				for (size_t k = 0; k < nSlot; ++k) dAcc[k](d[t][k].sum());
			}
		}
		std::vector<cplx> D(nSlot, cplx(0, 0));
		for (size_t k = 0; k < nSlot; ++k) D[k] = dAcc[k].sum();
		double dFlat = flatAcc.sum();

		// normalisation, pwaLikelihood.cc:254-273
		kahan<double> normAcc;
		const double nEvt = normFactor();
		const double twice = 2 * nEvt;
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned i = 0; i < nW[e]; ++i) {
					kahan<cplx> ndAcc;
					for (unsigned j = 0; j < nW[e]; ++j) {
						const cplx I = accM[mIdx(e, i, e, j)];
						normAcc(std::real((V[pIdx(r, e, i)] * std::conj(V[pIdx(r, e, j)])) * I));
						ndAcc(V[pIdx(r, e, j)] * std::conj(I));
					}
					D[pIdx(r, e, i)] += ndAcc.sum() * twice;
				}
		normAcc(flat2 * totAcc);
		dFlat += flat * twice * totAcc;

		// prior, pwaLikelihood.cc:278-297
		double prior = 0.;
		if (effPrior() == 1)
			for (unsigned r = 0; r < rank; ++r)
				for (unsigned e = 0; e < 2; ++e)
					for (unsigned w = 0; w < nW[e]; ++w) {
						const cplx v = V[pIdx(r, e, w)];
						const double rr = std::abs(v);
						const double cf = cauchyF(rr, cauchyWidth);
						const double fac = (1. / (rr * cf)) * cauchyD(rr, cauchyWidth);
						prior -= std::log(cf);
						D[pIdx(r, e, w)] -= cplx(fac * v.real(), fac * v.imag());
					}
		if (withGrad)
			toPar(D, dFlat, grad);
		if (fOut)
			*fOut = llAcc.sum() + nEvt * normAcc.sum() + prior;
	}

	// Analytic Hessian, pwaLikelihood.cc:639-859.  Output: nPars x nPars, row-major.
	void hessian(const double* par, double* H) const
	{
		std::vector<cplx> V;
		double flat;
		fromPar(par, V, flat);
		const double flat2 = flat * flat;
		const size_t nSlot = (size_t)rank * 2 * nWmax;
		// [slot i][slot j][3]
		std::vector<kahan<double> > hAcc(nSlot * nSlot * 3);
		std::vector<kahan<cplx> > flatTermsAcc(nSlot);
		kahan<double> hFlatAcc;
		for (unsigned long ev = 0; ev < nEvents; ++ev) {
			kahan<double> lAcc;
			std::vector<cplx> deriv(nSlot, cplx(0, 0));
			for (unsigned r = 0; r < rank; ++r) {
				for (unsigned e = 0; e < 2; ++e) {
					kahan<cplx> sAcc;
					const cplx* A = &amps[e][(size_t)ev * nW[e]];
					for (unsigned w = 0; w < nW[e]; ++w)
						sAcc(V[pIdx(r, e, w)] * A[w]);
					const cplx S = sAcc.sum();
					lAcc(std::norm(S));
					for (unsigned w = 0; w < nW[e]; ++w)
						deriv[pIdx(r, e, w)] = S;
				}
				for (unsigned e = 0; e < 2; ++e) {
					const cplx* A = &amps[e][(size_t)ev * nW[e]];
					for (unsigned w = 0; w < nW[e]; ++w)
						deriv[pIdx(r, e, w)] *= std::conj(A[w]);
				}
			}
			lAcc(flat2);
			const double factor = 2. / lAcc.sum();
			const double factor2 = factor * factor;
			for (unsigned ri = 0; ri < rank; ++ri)
				for (unsigned ei = 0; ei < 2; ++ei)
					for (unsigned wi = 0; wi < nW[ei]; ++wi) {
						const size_t si = pIdx(ri, ei, wi);
						for (unsigned rj = 0; rj < rank; ++rj)
							for (unsigned ej = 0; ej < 2; ++ej)
								for (unsigned wj = 0; wj < nW[ej]; ++wj) {
									const size_t sj = pIdx(rj, ej, wj);
									kahan<double>* h = &hAcc[(si * nSlot + sj) * 3];
									h[0](factor2 * deriv[sj].real() * deriv[si].real());
									h[1](factor2 * deriv[sj].imag() * deriv[si].real());
									h[2](factor2 * deriv[sj].imag() * deriv[si].imag());
									if (ri == rj and ei == ej) {
										const cplx u = std::conj(amps[ej][(size_t)ev * nW[ej] + wj]) *
										               amps[ei][(size_t)ev * nW[ei] + wi];
										h[0](-factor * u.real());
										h[1](-factor * u.imag());
										h[2](-factor * u.real());
									}
								}
						flatTermsAcc[si](factor2 * flat * deriv[si]);
					}
			hFlatAcc(factor2 * flat2 - factor);
		}
		std::vector<double> h(nSlot * nSlot * 3, 0.);
		for (size_t k = 0; k < h.size(); ++k) h[k] = hAcc[k].sum();
		std::vector<cplx> flatTerms(nSlot);
		for (size_t k = 0; k < nSlot; ++k) flatTerms[k] = flatTermsAcc[k].sum();
		double hFlat = hFlatAcc.sum();

		const double nEvt = normFactor();
		const double twice = 2 * nEvt;
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e)
				for (unsigned i = 0; i < nW[e]; ++i)
					for (unsigned j = 0; j < nW[e]; ++j) {
						const cplx I = accM[mIdx(e, i, e, j)];
						double* hh = &h[(pIdx(r, e, i) * nSlot + pIdx(r, e, j)) * 3];
						hh[0] += I.real() * twice;
						hh[1] += I.imag() * twice;
						hh[2] += I.real() * twice;
					}
		hFlat += twice * totAcc;

		if (effPrior() == 1)
			for (unsigned r = 0; r < rank; ++r)
				for (unsigned e = 0; e < 2; ++e)
					for (unsigned w = 0; w < nW[e]; ++w) {
						const cplx v = V[pIdx(r, e, w)];
						const double rr = std::abs(v);
						const double cf = cauchyF(rr, cauchyWidth), cd = cauchyD(rr, cauchyWidth),
						             cd2 = cauchyD2(rr, cauchyWidth);
						const double a1 = cd2 / (cf * rr * rr);
						const double a2 = cd * cd / (cf * cf * rr * rr);
						const double a3 = cd / (cf * rr);
						const double a4 = cd / (cf * rr * rr * rr);
						const double a124 = a1 - a2 - a4;
						const double re = v.real(), im = v.imag();
						double* hh = &h[(pIdx(r, e, w) * nSlot + pIdx(r, e, w)) * 3];
						hh[0] -= a124 * re * re + a3;
						hh[1] -= a124 * re * im;
						hh[2] -= a124 * im * im + a3;
					}

		std::fill(H, H + (size_t)nPars * nPars, 0.);
		for (unsigned ri = 0; ri < rank; ++ri)
			for (unsigned ei = 0; ei < 2; ++ei)
				for (unsigned wi = 0; wi < nW[ei]; ++wi) {
					const size_t si = pIdx(ri, ei, wi);
					const int r1 = mapRe[si], i1 = mapIm[si];
					if (r1 < 0 or pars[r1].fixed)
						continue;
					for (unsigned rj = 0; rj < rank; ++rj)
						for (unsigned ej = 0; ej < 2; ++ej)
							for (unsigned wj = 0; wj < nW[ej]; ++wj) {
								const size_t sj = pIdx(rj, ej, wj);
								const int r2 = mapRe[sj], i2 = mapIm[sj];
								if (r2 < 0 or pars[r2].fixed)
									continue;
								H[(size_t)r1 * nPars + r2] = h[(si * nSlot + sj) * 3 + 0];
								if (i2 >= 0)
									H[(size_t)r1 * nPars + i2] = h[(si * nSlot + sj) * 3 + 1];
								if (i1 >= 0)
									H[(size_t)i1 * nPars + r2] = h[(sj * nSlot + si) * 3 + 1];
								if (i1 >= 0 and i2 >= 0)
									H[(size_t)i1 * nPars + i2] = h[(si * nSlot + sj) * 3 + 2];
							}
					H[(size_t)r1 * nPars + nPars - 1] = flatTerms[si].real();
					H[(size_t)(nPars - 1) * nPars + r1] = flatTerms[si].real();
					if (i1 >= 0) {
						H[(size_t)i1 * nPars + nPars - 1] = flatTerms[si].imag();
						H[(size_t)(nPars - 1) * nPars + i1] = flatTerms[si].imag();
					}
				}
		H[(size_t)(nPars - 1) * nPars + nPars - 1] = hFlat;
	}

	// pwaLikelihood.cc:916-981: invert the free-parameter block (Gauss-Jordan with
	// partial pivoting, standing in for TMatrixT's LU inversion).
	bool covariance(const double* H, double* C) const
	{
		std::vector<unsigned> freeIdx;
		for (unsigned i = 0; i < nPars; ++i)
			if (not pars[i].fixed)
				freeIdx.push_back(i);
		const size_t n = freeIdx.size();
		std::vector<double> a(n * n), inv(n * n, 0.);
		for (size_t i = 0; i < n; ++i) {
			for (size_t j = 0; j < n; ++j)
				a[i * n + j] = H[(size_t)freeIdx[i] * nPars + freeIdx[j]];
			inv[i * n + i] = 1.;
		}
		for (size_t c = 0; c < n; ++c) {
			size_t piv = c;
			for (size_t r = c + 1; r < n; ++r)
				if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c]))
					piv = r;
			if (a[piv * n + c] == 0.)
				return false;
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
				if (r == c) continue;
				const double f = a[r * n + c];
				if (f == 0.) continue;
				for (size_t k = 0; k < n; ++k) {
					a[r * n + k] -= f * a[c * n + k];
					inv[r * n + k] -= f * inv[c * n + k];
				}
			}
		}
		std::fill(C, C + (size_t)nPars * nPars, 0.);
		for (size_t i = 0; i < n; ++i)
			for (size_t j = 0; j < n; ++j)
				C[(size_t)freeIdx[i] * nPars + freeIdx[j]] = inv[i * n + j];
		return true;
	}

	// pwaLikelihood.cc:984-1010
	void correctParamSigns(const double* par, double* out) const
	{
		std::vector<cplx> V;
		double flat;
		fromPar(par, V, flat);
		if (flat < 0)
			flat *= -1;
		for (unsigned r = 0; r < rank; ++r)
			for (unsigned e = 0; e < 2; ++e) {
				if (r >= nWmax)
					continue;
				const cplx anchor = V[pIdx(r, e, r)];
				if (anchor.real() < 0 and anchor.imag() == 0)
					for (unsigned w = 0; w < nW[e]; ++w)
						V[pIdx(r, e, w)] *= -1;
			}
		toPar(V, flat, out);
	}
};

// ampIntegralMatrix::integrate restated (ampIntegralMatrix.cc:299-488) over an
// in-memory amplitude array amps[wave][event][sub] (complex128 interleaved).
// weightStream holds the importance-sampling weights w in the order the
// reference reads its weight file: one value per event that passes the bin
// selection; each contributes 1/w.  inBin (optional) is the on-the-fly bin cut.
bool integrateImpl(OracleIntegral& I, unsigned nWaves, const char* const* names, const double* a,
                   unsigned long nEv, unsigned nSub, const double* weightStream, unsigned long nWeights,
                   const unsigned char* inBin, long maxNmbEvents)
{
	if (nWaves == 0 or nEv == 0 or nSub == 0)
		return false;
	if (I.waveNames.empty()) {
		I.nmbWaves = nWaves;
		for (unsigned i = 0; i < nWaves; ++i) I.waveNames.push_back(names[i]);
	} else {
		if (I.waveNames.size() != nWaves)
			return false;
		for (unsigned i = 0; i < nWaves; ++i)
			if (I.waveNames[i] != names[i])
				return false;
	}
	unsigned long nProc = (maxNmbEvents <= 0) ? nEv : std::min<unsigned long>(nEv, (unsigned long)maxNmbEvents);
	kahan<double> weightAcc;
	std::vector<kahan<cplx> > acc((size_t)nWaves * nWaves);
	std::vector<cplx> amp((size_t)nWaves * nSub);
	bool success = true;
	unsigned long counter = 0, wIdx = 0;
	const bool useWeight = (weightStream != nullptr);
	for (unsigned long ev = 0; ev < nProc; ++ev) {
		if (inBin and not inBin[ev])
			continue;
		++counter;
		double w = 1;
		if (useWeight) {
			if (wIdx >= nWeights) {
				success = false;
				break;
			}
			w = weightStream[wIdx++];
		}
		const double weight = 1 / w;
		weightAcc(weight);
		for (unsigned wv = 0; wv < nWaves; ++wv)
			for (unsigned s = 0; s < nSub; ++s) {
				const size_t k = ((size_t)wv * nEv + ev) * nSub + s;
				amp[(size_t)wv * nSub + s] = cplx(a[2 * k], a[2 * k + 1]);
			}
		for (unsigned i = 0; i < nWaves; ++i)
			for (unsigned j = 0; j < nWaves; ++j) {
				cplx val = 0;
				for (unsigned s = 0; s < nSub; ++s)
					val += amp[(size_t)i * nSub + s] * std::conj(amp[(size_t)j * nSub + s]);
				if (useWeight)
					val *= weight;
				acc[(size_t)i * nWaves + j](val);
			}
	}
	I.nmbEvents = counter;
	I.sums.assign((size_t)nWaves * nWaves, cplx(0, 0));
	const double weightNorm = weightAcc.sum() / (double)I.nmbEvents;
	for (size_t k = 0; k < I.sums.size(); ++k) {
		I.sums[k] = acc[k].sum();
		if (useWeight)
			I.sums[k] *= 1 / weightNorm;
	}
	return success;
}

// Shortest round-trip decimal of a double in the reference's "maxPrecisionDouble"
// spirit: 17 significant digits in scientific notation.
std::string fmtComplex(const cplx& c)
{
	std::ostringstream o;
	o << std::scientific << std::setprecision(std::numeric_limits<double>::max_digits10 - 1) << "(" << c.real()
	  << "," << c.imag() << ")";
	return o.str();
}

}  // namespace

extern "C" {

// ---------------- integral matrix ----------------
void* oracle_int_create() { return new OracleIntegral(); }
void oracle_int_destroy(void* h) { delete (OracleIntegral*)h; }
int oracle_int_set_wave_names(void* h, unsigned n, const char* const* names)
{
	OracleIntegral& I = *(OracleIntegral*)h;
	if (I.nmbWaves > 0) {
		if (n != I.nmbWaves) return 0;
		for (unsigned i = 0; i < n; ++i)
			if (I.waveNames[i] != names[i]) return 0;
		return 1;
	}
	I.waveNames.clear();
	for (unsigned i = 0; i < n; ++i) I.waveNames.push_back(names[i]);
	I.nmbWaves = n;
	I.sums.assign((size_t)n * n, cplx(0, 0));
	return 1;
}
int oracle_int_integrate(void* h, unsigned nWaves, const char* const* names, const double* amps, unsigned long nEv,
                         unsigned nSub, const double* weights, unsigned long nWeights, const unsigned char* inBin,
                         long maxNmbEvents)
{
	return integrateImpl(*(OracleIntegral*)h, nWaves, names, amps, nEv, nSub, weights, nWeights, inBin,
	                     maxNmbEvents) ? 1 : 0;
}
// ampIntegralMatrix.cc:279-297 (no compensation, as in the reference)
int oracle_int_add_event(void* h, const double* amps)
{
	OracleIntegral& I = *(OracleIntegral*)h;
	for (unsigned i = 0; i < I.nmbWaves; ++i)
		for (unsigned j = 0; j < I.nmbWaves; ++j)
			I.sums[(size_t)i * I.nmbWaves + j] +=
			    cplx(amps[2 * i], amps[2 * i + 1]) * std::conj(cplx(amps[2 * j], amps[2 * j + 1]));
	++I.nmbEvents;
	return 1;
}
void oracle_int_element(void* h, unsigned i, unsigned j, double* out)
{
	const cplx c = ((OracleIntegral*)h)->element(i, j);
	out[0] = c.real();
	out[1] = c.imag();
}
void oracle_int_raw(void* h, double* out)
{
	const OracleIntegral& I = *(OracleIntegral*)h;
	for (size_t k = 0; k < I.sums.size(); ++k) {
		out[2 * k] = I.sums[k].real();
		out[2 * k + 1] = I.sums[k].imag();
	}
}
void oracle_int_set_raw(void* h, const double* in)
{
	OracleIntegral& I = *(OracleIntegral*)h;
	for (size_t k = 0; k < I.sums.size(); ++k) I.sums[k] = cplx(in[2 * k], in[2 * k + 1]);
}
unsigned long oracle_int_nmb_events(void* h) { return ((OracleIntegral*)h)->nmbEvents; }
void oracle_int_set_nmb_events(void* h, unsigned long n) { ((OracleIntegral*)h)->nmbEvents = n; }
unsigned oracle_int_nmb_waves(void* h) { return ((OracleIntegral*)h)->nmbWaves; }
// operator+= (ampIntegralMatrix.cc:125-142): elements matched by wave name
int oracle_int_add(void* h, void* o)
{
	OracleIntegral& A = *(OracleIntegral*)h;
	const OracleIntegral& B = *(OracleIntegral*)o;
	if (A.nmbWaves != B.nmbWaves) return 0;
	std::vector<int> idx(A.nmbWaves);
	for (unsigned i = 0; i < A.nmbWaves; ++i) {
		idx[i] = B.waveIndex(A.waveNames[i]);
		if (idx[i] < 0) return 0;
	}
	for (unsigned i = 0; i < A.nmbWaves; ++i)
		for (unsigned j = 0; j < A.nmbWaves; ++j)
			A.sums[(size_t)i * A.nmbWaves + j] += B.sums[(size_t)idx[i] * B.nmbWaves + idx[j]];
	A.nmbEvents += B.nmbEvents;
	return 1;
}
// readAscii (ampIntegralMatrix.cc:527-569)
int oracle_int_read_ascii(void* h, const char* path)
{
	OracleIntegral& I = *(OracleIntegral*)h;
	std::ifstream in(path);
	if (not in) return 0;
	unsigned nw;
	unsigned long ne;
	if (not(in >> nw >> ne)) return 0;
	unsigned nr, nc;
	if (not(in >> nr >> nc)) return 0;
	I.nmbWaves = nw;
	I.nmbEvents = ne;
	I.sums.assign((size_t)nr * nc, cplx(0, 0));
	for (unsigned i = 0; i < nr; ++i)
		for (unsigned j = 0; j < nc; ++j) {
			cplx v;
			if (not(in >> v) or in.eof()) return 0;
			I.sums[(size_t)i * nc + j] = v;
		}
	I.waveNames.assign(nw, std::string());
	unsigned mapSize;
	in >> mapSize;
	if (mapSize != nw) return 0;
	while (mapSize > 0 and in) {
		std::string name;
		unsigned idx;
		if (not(in >> name >> idx)) return 0;
		if (idx >= nw) return 0;
		I.waveNames[idx] = name;
		--mapSize;
	}
	return 1;
}
// writeAscii (ampIntegralMatrix.cc:502-524); the wave-name map is written to
// the file (the reference sends it to stdout by mistake, :521).
int oracle_int_write_ascii(void* h, const char* path)
{
	const OracleIntegral& I = *(OracleIntegral*)h;
	std::ofstream out(path);
	if (not out) return 0;
	out << I.nmbWaves << "\n" << I.nmbEvents << "\n" << I.nmbWaves << " " << I.nmbWaves << "\n";
	for (unsigned i = 0; i < I.nmbWaves; ++i) {
		for (unsigned j = 0; j < I.nmbWaves; ++j) out << fmtComplex(I.sums[(size_t)i * I.nmbWaves + j]) << "\t";
		out << "\n";
	}
	out << I.waveNames.size() << "\n";
	for (unsigned i = 0; i < I.nmbWaves; ++i) out << I.waveNames[i] << " " << i << "\n";
	return 1;
}
int oracle_int_wave_name(void* h, unsigned i, char* buf, unsigned len)
{
	const OracleIntegral& I = *(OracleIntegral*)h;
	if (i >= I.waveNames.size() or len == 0) return 0;
	std::snprintf(buf, len, "%s", I.waveNames[i].c_str());
	return 1;
}

// ---------------- likelihood ----------------
void* oracle_lik_create() { return new OracleLikelihood(); }
void oracle_lik_destroy(void* h) { delete (OracleLikelihood*)h; }
void oracle_lik_set_options(void* h, int useNormalizedAmps, int priorType, double cauchyWidth)
{
	OracleLikelihood& L = *(OracleLikelihood*)h;
	L.useNormalizedAmps = useNormalizedAmps != 0;
	L.priorType = priorType;
	L.cauchyWidth = cauchyWidth;
}
void oracle_lik_set_shard(void* h, unsigned long totalEvents, int root)
{
	OracleLikelihood& L = *(OracleLikelihood*)h;
	L.shardSet = true;
	L.shardTotal = totalEvents;
	L.shardRoot = root != 0;
}
int oracle_lik_set_otf_binning(void* h, unsigned nVars, const double* lower, const double* upper,
                               const double* const* vars, unsigned long nFile)
{
	return ((OracleLikelihood*)h)->setOtf(nVars, lower, upper, vars, nFile) ? 1 : 0;
}
unsigned long oracle_lik_otf_selected(void* h) { return ((OracleLikelihood*)h)->otfIdx.size(); }
int oracle_lik_init(void* h, unsigned n, const char* const* names, const int* refl, const double* thres,
                    unsigned rank, double massBinCenter)
{
	return ((OracleLikelihood*)h)->init(n, names, refl, thres, rank, massBinCenter) ? 1 : 0;
}
int oracle_lik_add_norm_integral(void* h, void* I)
{
	return ((OracleLikelihood*)h)->addNormIntegral(*(OracleIntegral*)I) ? 1 : 0;
}
int oracle_lik_add_acc_integral(void* h, void* I, unsigned long override_)
{
	return ((OracleLikelihood*)h)->addAccIntegral(*(OracleIntegral*)I, override_) ? 1 : 0;
}
int oracle_lik_add_amplitude(void* h, const char* name, const double* amps, unsigned long n)
{
	return ((OracleLikelihood*)h)->addAmplitude(name, amps, n) ? 1 : 0;
}
int oracle_lik_finish_init(void* h) { return ((OracleLikelihood*)h)->finishInit() ? 1 : 0; }
unsigned oracle_lik_nmb_pars(void* h) { return ((OracleLikelihood*)h)->nPars; }
unsigned oracle_lik_nmb_pars_fixed(void* h)
{
	unsigned n = 0;
	for (auto& p : ((OracleLikelihood*)h)->pars) n += p.fixed ? 1 : 0;
	return n;
}
int oracle_lik_par_fixed(void* h, unsigned i) { return ((OracleLikelihood*)h)->pars[i].fixed ? 1 : 0; }
// fitParameter::parName, pwaLikelihood.cc:107-122
int oracle_lik_par_name(void* h, unsigned i, char* buf, unsigned len)
{
	const ParInfo& p = ((OracleLikelihood*)h)->pars[i];
	std::ostringstream o;
	o << "V";
	if (p.waveName != "flat") o << p.rank;
	o << "_" << p.waveName << (p.realPart ? "_RE" : "_IM");
	std::snprintf(buf, len, "%s", o.str().c_str());
	return 1;
}
// nmbWaves(reflectivity), pwaLikelihood.cc:1013-1022
unsigned oracle_lik_nmb_waves(void* h, int refl)
{
	const OracleLikelihood& L = *(OracleLikelihood*)h;
	if (refl == 0) return L.nW[0] + L.nW[1];
	return refl > 0 ? L.nW[1] : L.nW[0];
}
double oracle_lik_tot_acc(void* h) { return ((OracleLikelihood*)h)->totAcc; }
void oracle_lik_fdf(void* h, const double* par, double* f, double* grad, unsigned nThreads)
{
	((OracleLikelihood*)h)->fdf(par, f, grad, true, nThreads);
}
double oracle_lik_doeval(void* h, const double* par, unsigned nThreads)
{
	double f;
	((OracleLikelihood*)h)->fdf(par, &f, nullptr, false, nThreads);
	return f;
}
void oracle_lik_gradient(void* h, const double* par, double* grad, unsigned nThreads)
{
	((OracleLikelihood*)h)->fdf(par, nullptr, grad, true, nThreads);
}
void oracle_lik_hessian(void* h, const double* par, double* H) { ((OracleLikelihood*)h)->hessian(par, H); }
int oracle_lik_covariance(void* h, const double* H, double* C) { return ((OracleLikelihood*)h)->covariance(H, C) ? 1 : 0; }
void oracle_lik_correct_param_signs(void* h, const double* par, double* out)
{
	((OracleLikelihood*)h)->correctParamSigns(par, out);
}
// integral matrices in likelihood order [refl][wave] x [refl][wave], plus flat
// slot if withFlat (pwaLikelihood.cc:1577-1618)
void oracle_lik_integral_matrices(void* h, double* norm, double* acc, double* ps, int withFlat)
{
	const OracleLikelihood& L = *(OracleLikelihood*)h;
	const unsigned nw = L.nW[0] + L.nW[1];
	const unsigned sz = nw + (withFlat ? 1 : 0);
	std::fill(norm, norm + 2 * (size_t)sz * sz, 0.);
	std::fill(acc, acc + 2 * (size_t)sz * sz, 0.);
	unsigned ii = 0;
	for (unsigned e1 = 0; e1 < 2; ++e1)
		for (unsigned i = 0; i < L.nW[e1]; ++i, ++ii) {
			ps[ii] = L.phaseSpaceIntegral[e1 * L.nWmax + i];
			unsigned jj = 0;
			for (unsigned e2 = 0; e2 < 2; ++e2)
				for (unsigned j = 0; j < L.nW[e2]; ++j, ++jj) {
					const cplx n = L.normM[L.mIdx(e1, i, e2, j)], a = L.accM[L.mIdx(e1, i, e2, j)];
					norm[2 * ((size_t)ii * sz + jj)] = n.real();
					norm[2 * ((size_t)ii * sz + jj) + 1] = n.imag();
					acc[2 * ((size_t)ii * sz + jj)] = a.real();
					acc[2 * ((size_t)ii * sz + jj) + 1] = a.imag();
				}
		}
	if (withFlat) {
		norm[2 * ((size_t)nw * sz + nw)] = 1.;
		acc[2 * ((size_t)nw * sz + nw)] = L.totAcc;
		ps[nw] = 1.;
	}
}

}  // extern "C"
