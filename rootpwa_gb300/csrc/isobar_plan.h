// isobar_plan.h -- host side of the three-body isobar amplitudes: spin
// algebra and the wave plan that the per-event arithmetic (isobar_math.cuh)
// reads.  Header-only so that the CPU tests can compile the plan builder and
// the per-event arithmetic together without the CUDA runtime.
//
// Every spin, spin projection and orbital angular momentum is an integer in
// units of 1/2 (2J, 2M, 2L), as in the reference (utilities/spinUtils.hpp).
#pragma once

#include "../../include/pwa_gb300.h"
#include "isobar_math.cuh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <tuple>
#include <vector>

namespace pwa {
namespace iso {

inline double factorial(int n)
{
	double r = 1.0;
	for (int i = 2; i <= n; ++i)
		r *= i;
	return r;
}

// (j1 m1 j2 m2 | J M) by Racah's formula, Condon-Shortley phase
// (replaces clebschGordanCoeff, utilities/spinUtils.hpp:241-330)
inline double clebschGordan(int j1, int m1, int j2, int m2, int J, int M)
{
	auto ok = [](int j, int m) { return j >= 0 && std::abs(m) <= j && ((j - m) & 1) == 0; };
	if (!ok(j1, m1) || !ok(j2, m2) || !ok(J, M) || m1 + m2 != M)
		return 0.0;
	if (J < std::abs(j1 - j2) || J > j1 + j2 || ((j1 + j2 + J) & 1))
		return 0.0;
	const int a = (j1 + j2 - J) / 2, b = (j1 - m1) / 2, c = (j2 + m2) / 2;
	const int d = (J - j2 + m1) / 2, e = (J - j1 - m2) / 2;
	double sum = 0.0;
	for (int k = std::max(0, std::max(-d, -e)); k <= std::min(a, std::min(b, c)); ++k)
		sum += ((k & 1) ? -1.0 : 1.0) /
		       (factorial(k) * factorial(a - k) * factorial(b - k) * factorial(c - k) * factorial(d + k) * factorial(e + k));
	const double tri = (J + 1) * factorial((J + j1 - j2) / 2) * factorial((J - j1 + j2) / 2) * factorial(a) /
	                   factorial((j1 + j2 + J) / 2 + 1);
	const double proj = factorial((J + M) / 2) * factorial((J - M) / 2) * factorial(b) * factorial((j1 + m1) / 2) *
	                    factorial((j2 - m2) / 2) * factorial(c);
	return std::sqrt(tri * proj) * sum;
}

// Wigner's formula: d^j_{m n}(theta) as terms coef cos^a(theta/2) sin^b(theta/2)
// (replaces dFunction, utilities/dFunction.hpp:52-170)
inline void wignerTerms(int j, int m, int n, std::vector<DTerm>& out)
{
	const int jpm = (j + m) / 2, jmm = (j - m) / 2, jpn = (j + n) / 2, jmn = (j - n) / 2;
	const int d = (m - n) / 2;
	const double root = std::sqrt(factorial(jpm) * factorial(jmm) * factorial(jpn) * factorial(jmn));
	for (int s = std::max(0, -d); s <= std::min(jpn, jmm); ++s) {
		const double coef = (((d + s) & 1) ? -1.0 : 1.0) * root /
		                    (factorial(jpn - s) * factorial(s) * factorial(d + s) * factorial(jmm - s));
		out.push_back(DTerm{coef, jpn + jmm - 2 * s, d + 2 * s});
	}
}

inline double wignerD(int j, int m, int n, double theta)
{
	std::vector<DTerm> t;
	wignerTerms(j, m, n, t);
	return dEval(t.data(), 0, (int)t.size(), std::cos(0.5 * theta), std::sin(0.5 * theta));
}

// Blatt-Weisskopf denominators.  x h_l(x) = (-i)^(l+1) e^{ix} sum_k a_k (i/2x)^k
// with a_k = (l+k)! / (k! (l-k)!) (the reverse Bessel polynomial), so
// |x h_l(x)|^2 z^l = P_l(z), z = x^2, with integer coefficients
// [z^(l-m)] P_l = c_m / 4^m, c_m = sum_k (-1)^(m-k) a_{2m-k} a_k.  F_L^2 is
// P_l(1) z^l / P_l(z): 1 at q = 0.1973 GeV/c, l = 0 .. 7 (replaces the table
// in utilities/physUtils.hpp:200-262).
inline void barrierPolynomials(double poly[8][8], double norm[8])
{
	for (int l = 0; l < 8; ++l) {
		int64_t a[16] = {0};
		for (int k = 0; k <= l; ++k) {
			int64_t v = 1;  // (l+k)! / (k! (l-k)!)
			for (int i = l - k + 1; i <= l + k; ++i)
				v *= i;
			for (int i = 2; i <= k; ++i)
				v /= i;
			a[k] = v;
		}
		for (int k = 0; k < 8; ++k)
			poly[l][k] = 0.0;
		for (int m = 0; m <= l; ++m) {
			int64_t c = 0;
			for (int k = 0; k <= 2 * m; ++k)
				c += (((m - k) & 1) ? -1 : 1) * a[2 * m - k] * a[k];
			poly[l][l - m] = (double)(c / ((int64_t)1 << (2 * m)));
		}
		double s = 0.0;
		for (int k = 0; k <= l; ++k)
			s += poly[l][k];
		norm[l] = s;
	}
}

// checks a wave; returns an empty string or the reason it is refused
inline std::string checkWave(const pwa_isobar_wave& w, bool reflBasis)
{
	auto even = [](int x) { return (x & 1) == 0; };
	if (w.J < 0 || w.J > kMaxSpin || w.isobarJ < 0 || w.isobarJ > kMaxSpin)
		return "spins must be in 0 .. 16 (units of 1/2)";
	if (!even(w.J) || !even(w.isobarJ) || !even(w.L) || !even(w.S) || !even(w.isobarL) || !even(w.isobarS) ||
	    !even(w.M))
		return "three spinless final-state particles: every spin and projection must be an integer (even in units of 1/2)";
	if (std::abs(w.M) > w.J)
		return "|M| > J";
	if (reflBasis && w.M < 0)
		return "the reflectivity basis needs M >= 0";
	if ((w.P != 1 && w.P != -1) || (w.refl != 1 && w.refl != -1))
		return "parity and reflectivity must be +1 or -1";
	if (w.L < 0 || w.L > kMaxL || w.isobarL < 0 || w.isobarL > kMaxL)
		return "orbital angular momenta must be in 0 .. 14 (units of 1/2)";
	if (w.S < 0 || w.S > 2 * kMaxSpin || w.isobarS < 0 || w.isobarS > 2 * kMaxSpin)
		return "coupled spins out of range";
	const int a = w.isobarDaughter1, b = w.isobarDaughter2, c = w.bachelor;
	if (a < 0 || b < 0 || c < 0 || a > 2 || b > 2 || c > 2 || a == b || a == c || b == c)
		return "isobar daughters and bachelor must be three distinct final-state slots 0..2";
	if (w.massDependence < kMassFlat || w.massDependence > kMassKPiSPalano)
		return "unknown mass dependence";
	if (w.massDependence == kMassBinned && !(w.binLower <= w.binUpper))
		return "a mass bin needs lower <= upper";
	if (w.massDependence >= kMassRelBw && w.massDependence <= kMassF0980Bw && !(w.isobarMass > 0 && w.isobarWidth > 0))
		return "a Breit-Wigner needs a positive mass and width";
	return std::string();
}

struct Plan {
	std::vector<WaveDev> waves;
	std::vector<int32_t> order;
	std::vector<LamTerm> lams;
	std::vector<DTerm> dterms;
	double bfPoly[8][8];
	double bfNorm[8];
	float bfPolyF[8][8];            // FP32 copies (complex64 mode)
	float bfNormF[8];
	std::vector<int32_t> perms;     // the six permutations of three slots
	std::vector<SymTerm> terms;
	double masses[3] = {0.0, 0.0, 0.0}, beamMass = 0.0;
	int32_t spaceInversion = 0, reflection = 0, canonical = 0;

	PlanView view() const
	{
		PlanView v{};
		v.waves = waves.data();
		v.order = order.data();
		v.lams = lams.data();
		v.dterms = dterms.data();
		v.bfPoly = &bfPoly[0][0];
		v.bfNorm = bfNorm;
		v.bfPolyF = &bfPolyF[0][0];
		v.bfNormF = bfNormF;
		v.perms = perms.data();
		v.terms = terms.data();
		v.nWaves = (uint32_t)waves.size();
		for (int i = 0; i < 3; ++i)
			v.masses[i] = masses[i];
		v.beamMass = beamMass;
		v.spaceInversion = spaceInversion;
		v.reflection = reflection;
		v.canonical = canonical;
		return v;
	}
};

// FP32 copies of the plan's constants for the complex64 kernel, whose
// per-wave arithmetic is FP32 (converting FP64 constants there would put
// each conversion on the FP64 pipe); M^2 - m^2 of the Breit-Wigner
// denominators takes M as an FP32 hi + lo pair
inline void fillFp32Copies(Plan& plan)
{
	for (DTerm& t : plan.dterms)
		t.coefF = (float)t.coef;
	for (LamTerm& t : plan.lams) {
		t.cPlusF = (float)t.cPlus;
		t.cMinusF = (float)t.cMinus;
	}
	for (SymTerm& t : plan.terms)
		t.factorF = (float)t.factor;
	for (int i = 0; i < 8; ++i) {
		for (int k = 0; k < 8; ++k)
			plan.bfPolyF[i][k] = (float)plan.bfPoly[i][k];
		plan.bfNormF[i] = (float)plan.bfNorm[i];
	}
	for (WaveDev& w : plan.waves) {
		w.q0Zero = w.q0 == 0.0 ? 1 : 0;
		w.m0F = (float)w.m0;
		w.g0F = (float)w.g0;
		w.q0F = (float)w.q0;
		w.f2q0F = (float)w.f2q0;
		w.maF = (float)w.ma;
		w.mbF = (float)w.mb;
		w.q02F = (float)w.q02;
		const double M = w.massDep == kMassF0980Flatte ? kFlatteM0 : w.m0;
		w.dmHi = (float)M;
		w.dmLo = (float)(M - (double)w.dmHi);
	}
}

// a permutation of the three final-state slots: slot i takes particle p[i]
typedef std::vector<int> Perm;
struct Term {
	Perm perm;
	double factor;
};

// index of a permutation in the lexicographic list of the six (the kernel's table)
inline int permIndex(const Perm& p)
{
	int q[3] = {0, 1, 2}, k = 0;
	do {
		if (q[0] == p[0] && q[1] == p[1] && q[2] == p[2])
			return k;
		++k;
	} while (std::next_permutation(q, q + 3));
	return -1;
}

// permutations that only exchange particles of equal species, factor
// 1/sqrt(number of terms) = 1/sqrt(prod n_k!)
// (isobarDecayTopology::getBoseSymmetrization, isobarDecayTopology.cc:638-670)
inline std::vector<Term> boseTerms(const int32_t species[3], bool bose)
{
	std::vector<Term> out;
	int p[3] = {0, 1, 2};
	if (!bose)
		return {Term{Perm(p, p + 3), 1.0}};
	do {
		if (species[p[0]] == species[0] && species[p[1]] == species[1] && species[p[2]] == species[2])
			out.push_back(Term{Perm(p, p + 3), 1.0});
	} while (std::next_permutation(p, p + 3));
	for (Term& t : out)
		t.factor = 1.0 / std::sqrt((double)out.size());
	return out;
}

// spinStatesCanCouple(j1, m1, j2, m2, J, M) (utilities/spinUtils.hpp:167):
// valid projections, triangle rule, M = m1 + m2
inline bool canCouple(int j1, int m1, int j2, int m2, int J, int M)
{
	auto ok = [](int j, int m) { return j >= 0 && std::abs(m) <= j && ((j - m) & 1) == 0; };
	return ok(j1, m1) && ok(j2, m2) && ok(J, M) && J >= std::abs(j1 - j2) && J <= j1 + j2 &&
	       ((j1 + j2 - J) & 1) == 0 && M == m1 + m2;
}

// final-state isospins for isospin symmetrisation (all doubled)
struct FsIsospin {
	int32_t I[3], I3[3], P[3];
};

// isobarDecayTopology::getIsospinSymmetrization (isobarDecayTopology.cc:505-630)
// for X -> isobar(a, b) + bachelor c: all permutations within groups of
// final-state particles of equal isospin and parity (spins are 0), ordered
// like getAllGroupPermutations (:889-923: the last group's permutation
// outermost); against every accepted permutation, one that exchanges
// particles of equal species or two particles of one vertex is dropped; the
// permuted isospin projections must couple at both vertices; the factor is
// the product of both vertices' isospin Clebsch-Gordan coefficients over
// sqrt(number of terms), or 1 for a single term (isobarAmplitude.cc:276-279).
inline std::vector<Term> isospinTerms(const pwa_isobar_wave& w, const int32_t species[3], const FsIsospin& fs)
{
	// groups of equal (I, P), in order of first appearance
	std::vector<std::vector<int>> groups;
	std::vector<std::pair<int, int>> keys;
	for (int i = 0; i < 3; ++i) {
		const std::pair<int, int> k(fs.I[i], fs.P[i]);
		auto it = std::find(keys.begin(), keys.end(), k);
		if (it == keys.end()) {
			keys.push_back(k);
			groups.push_back({i});
		} else {
			groups[it - keys.begin()].push_back(i);
		}
	}
	// all products of within-group permutations, the last group outermost
	std::vector<std::vector<std::vector<int>>> combos{{}};
	for (const std::vector<int>& g : groups) {
		std::vector<int> cur = g;
		std::sort(cur.begin(), cur.end());
		std::vector<std::vector<int>> gp;
		do
			gp.push_back(cur);
		while (std::next_permutation(cur.begin(), cur.end()));
		std::vector<std::vector<std::vector<int>>> next;
		for (const std::vector<int>& c : gp)
			for (const std::vector<std::vector<int>>& sub : combos) {
				std::vector<std::vector<int>> e = sub;
				e.push_back(c);
				next.push_back(e);
			}
		combos.swap(next);
	}
	const int a = w.isobarDaughter1, b = w.isobarDaughter2, c = w.bachelor;
	int vertexOf[3];
	vertexOf[a] = vertexOf[b] = 1;
	vertexOf[c] = 0;
	int I3X = 0;
	for (int i = 0; i < 3; ++i)
		I3X += fs.I3[i];
	std::vector<Term> acc;
	for (const std::vector<std::vector<int>>& combo : combos) {
		Perm p(3);
		for (size_t gi = 0; gi < groups.size(); ++gi)
			for (size_t k = 0; k < groups[gi].size(); ++k)
				p[groups[gi][k]] = combo[gi][k];
		bool drop = false;
		for (const Term& q : acc) {
			for (int i = 0; i < 3 && !drop; ++i) {
				if (q.perm[i] == p[i])
					continue;
				if (species[q.perm[i]] == species[p[i]]) {
					drop = true;
					break;
				}
				for (int j = i + 1; j < 3; ++j)
					if (q.perm[j] != p[j] && vertexOf[q.perm[i]] == vertexOf[q.perm[j]] &&
					    vertexOf[q.perm[i]] == vertexOf[p[i]] && vertexOf[p[i]] == vertexOf[p[j]]) {
						drop = true;
						break;
					}
			}
			if (drop)
				break;
		}
		if (drop)
			continue;
		int I3[3];
		for (int i = 0; i < 3; ++i)
			I3[i] = fs.I3[p[i]];
		const int I3iso = I3[a] + I3[b];
		int d1 = w.isobarIsospin, d1p = I3iso, d2 = fs.I[c], d2p = I3[c];
		if (w.bachelorFirst) {
			std::swap(d1, d2);
			std::swap(d1p, d2p);
		}
		if (!canCouple(fs.I[a], I3[a], fs.I[b], I3[b], w.isobarIsospin, I3iso) ||
		    !canCouple(d1, d1p, d2, d2p, w.isospin, I3X))
			continue;
		const double f = clebschGordan(d1, d1p, d2, d2p, w.isospin, I3X) *
		                 clebschGordan(fs.I[a], I3[a], fs.I[b], I3[b], w.isobarIsospin, I3iso);
		acc.push_back(Term{p, f});
	}
	if (acc.size() == 1)
		acc[0].factor = 1.0;
	else
		for (Term& t : acc)
			t.factor /= std::sqrt((double)acc.size());
	return acc;
}

// isobarAmplitude::initSymTermMaps (isobarAmplitude.cc:265-330): every
// isospin term combined with every Bose term, map[i] = bose[iso[i]], factor
// iso * bose
inline std::vector<Term> symTerms(const pwa_isobar_wave& w, const int32_t species[3], bool bose,
                                  const FsIsospin* isospin)
{
	const std::vector<Term> iso = isospin ? isospinTerms(w, species, *isospin) : std::vector<Term>{Term{{0, 1, 2}, 1.0}};
	const std::vector<Term> bt = boseTerms(species, bose);
	std::vector<Term> out;
	for (const Term& ti : iso)
		for (const Term& tb : bt) {
			Perm m(3);
			for (int i = 0; i < 3; ++i)
				m[i] = tb.perm[ti.perm[i]];
			out.push_back(Term{m, ti.factor * tb.factor});
		}
	return out;
}

// canonical formalism (isobarCanonicalAmplitude::twoBodyDecayAmplitude,
// isobarCanonicalAmplitude.cc:118-190): for each spin projection m of the
// isobar, X vertex sqrt(4 pi) (s1 m1 s2 m2 | S m) F_L sum_mL C(mL) Y_L^mL and
// isobar vertex sqrt(4 pi) (0 0 0 0 | S' 0) F_l (l m S' 0 | j m) Y_l^m.  The
// (L mL S m | J +-M) couplings vanish unless mL = +-M - m, so the sum over mL
// keeps two terms; sqrt(4 pi) Y_L^mu = sqrt(2L+1) e^{i mu phi} d^L_{mu 0}.
inline void addCanonicalTerms(const pwa_isobar_wave& s, bool reflBasis, Plan& plan)
{
	const int J = s.J, M = s.M, L = s.L, S = s.S, j = s.isobarJ, l = s.isobarL, Si = s.isobarS;
	for (int m = -j; m <= j; m += 2) {
		const int s1 = s.bachelorFirst ? 0 : j, m1 = s.bachelorFirst ? 0 : m;
		const int s2 = s.bachelorFirst ? j : 0, m2 = s.bachelorFirst ? m : 0;
		const double ss = clebschGordan(s1, m1, s2, m2, S, m);
		const double iso = std::sqrt(l + 1.0) * clebschGordan(0, 0, 0, 0, Si, 0) * clebschGordan(l, m, Si, 0, j, m);
		if (ss == 0.0 || iso == 0.0 || std::abs(m) > l)
			continue;
		double cP = 0.0, cM = 0.0;
		const int mP = M - m, mM = -M - m;
		if (reflBasis) {
			const int f = s.refl * s.P * ((((J - M) / 2) & 1) ? -1 : 1);
			if (M == 0) {
				if (f != +1)
					cP = clebschGordan(L, mP, S, m, J, 0);
			} else {
				cP = clebschGordan(L, mP, S, m, J, M) / std::sqrt(2.0);
				cM = -f * clebschGordan(L, mM, S, m, J, -M) / std::sqrt(2.0);
			}
		} else {
			cP = clebschGordan(L, mP, S, m, J, M);
		}
		if (std::abs(mP) > L)
			cP = 0.0;
		if (std::abs(mM) > L)
			cM = 0.0;
		if (cP == 0.0 && cM == 0.0)
			continue;
		const double c = std::sqrt(L + 1.0) * ss * iso;
		LamTerm t{};
		t.lamIso = m;
		t.plus0 = (int32_t)plan.dterms.size();
		if (cP != 0.0)
			wignerTerms(L, mP, 0, plan.dterms);
		t.plus1 = (int32_t)plan.dterms.size();
		t.minus0 = t.plus1;
		if (cM != 0.0)
			wignerTerms(L, mM, 0, plan.dterms);
		t.minus1 = (int32_t)plan.dterms.size();
		t.iso0 = t.minus1;
		wignerTerms(l, m, 0, plan.dterms);
		t.iso1 = (int32_t)plan.dterms.size();
		t.mPlus = mP;
		t.mMinus = mM;
		t.cPlus = c * cP;
		t.cMinus = c * cM;
		plan.lams.push_back(t);
	}
}

// wave plan of isobarHelicityAmplitude::twoBodyDecayAmplitude /
// twoBodyDecayAmplitudeSum (isobarHelicityAmplitude.cc:130-195,
// isobarAmplitude.cc:206-262) for every wave: the sum over the isobar's
// helicities with the Clebsch-Gordan couplings, sqrt(2L+1) norms
// (angMomNormFactor, physUtils.hpp:159-166) and the reflectivity-basis
// combination (dFunction.hpp DFunctionReflConj) folded into coefficients.
// returns an empty string, or why a wave cannot be evaluated with these
// final-state masses
inline std::string buildPlan(const std::vector<pwa_isobar_wave>& specs, const double masses[3],
                             const int32_t species[3], double beamMass, bool reflBasis, bool bose,
                             bool spaceInversion, bool reflection, bool canonical, const FsIsospin* isospin,
                             Plan& plan)
{
	plan.canonical = canonical ? 1 : 0;
	for (int i = 0; i < 3; ++i)
		plan.masses[i] = masses[i];
	plan.beamMass = beamMass;
	plan.spaceInversion = spaceInversion ? 1 : 0;
	plan.reflection = reflection ? 1 : 0;
	plan.waves.clear();
	plan.lams.clear();
	plan.dterms.clear();
	plan.terms.clear();
	barrierPolynomials(plan.bfPoly, plan.bfNorm);
	plan.perms.clear();
	{
		int q[3] = {0, 1, 2};
		do
			plan.perms.insert(plan.perms.end(), q, q + 3);
		while (std::next_permutation(q, q + 3));
	}
	std::vector<std::tuple<int, int, int, int>> topoKeys;
	for (const pwa_isobar_wave& s : specs) {
		WaveDev w{};
		w.a = s.isobarDaughter1;
		w.b = s.isobarDaughter2;
		w.c = s.bachelor;
		w.bachelorFirst = s.bachelorFirst ? 1 : 0;
		w.M = s.M;
		w.LX = s.L;
		w.LI = s.isobarL;
		w.massDep = s.massDependence;
		w.m0 = s.massDependence == kMassBinned ? s.binLower : s.isobarMass;
		w.g0 = s.massDependence == kMassBinned ? s.binUpper : s.isobarWidth;
		w.ma = masses[w.a];
		w.mb = masses[w.b];
		w.f2q0 = 1.0;
		for (int k = 0; k < 10; ++k)
			w.mdp[k] = s.massDepParams[k];
		w.q02 = breakup2(s.isobarMass, w.ma, w.mb);
		if (s.massDependence == kMassRelBw) {
			// the PWA2000 rule q0 = sqrt|q0^2| (massDependence.cc:268-270)
			w.q0 = std::sqrt(std::fabs(w.q02));
			const PlanView v = plan.view();
			w.f2q0 = barrierF2(v, s.isobarL, w.q0);
		} else if (s.massDependence == kMassRhoBw || s.massDependence == kMassF0980Bw) {
			// the reference refuses a resonance mass below the daughters' threshold
			if (!(w.q02 > 0.0))
				return "wave " + std::to_string(plan.waves.size()) +
				       ": the isobar mass is below the threshold of its daughters";
			w.q0 = std::sqrt(w.q02);
		}
		w.term0 = (int32_t)plan.terms.size();
		for (const Term& t : symTerms(s, species, bose, isospin))
			if (t.factor != 0.0)  // zero terms (a vanishing isospin coupling) only enter the normalisation
				plan.terms.push_back(SymTerm{permIndex(t.perm), 0.f, t.factor});
		w.term1 = (int32_t)plan.terms.size();
		const std::tuple<int, int, int, int> key(w.a, w.b, w.c, w.bachelorFirst);
		auto it = std::find(topoKeys.begin(), topoKeys.end(), key);
		w.topo = (int32_t)(it - topoKeys.begin());
		if (it == topoKeys.end())
			topoKeys.push_back(key);
		// reflectivity combination of the X vertex
		double wPlus = 1.0, wMinus = 0.0;
		bool zero = false;
		if (reflBasis) {
			const int f = s.refl * s.P * ((((s.J - s.M) / 2) & 1) ? -1 : 1);
			if (s.M == 0)
				zero = (f == +1);
			else {
				wPlus = 1.0 / std::sqrt(2.0);
				wMinus = -f / std::sqrt(2.0);
			}
		}
		w.lam0 = (int32_t)plan.lams.size();
		if (canonical) {
			addCanonicalTerms(s, reflBasis, plan);
			w.lam1 = (int32_t)plan.lams.size();
			plan.waves.push_back(w);
			continue;
		}
		for (int lamIso = -s.isobarJ; lamIso <= s.isobarJ && !zero; lamIso += 2) {
			// X -> daughter 1 + daughter 2 with helicities (l1, l2), spins (s1, s2)
			const int s1 = s.bachelorFirst ? 0 : s.isobarJ, l1 = s.bachelorFirst ? 0 : lamIso;
			const int s2 = s.bachelorFirst ? s.isobarJ : 0, l2 = s.bachelorFirst ? lamIso : 0;
			const int lam = l1 - l2;
			if (std::abs(lam) > s.J)
				continue;
			const double cgX = clebschGordan(s.L, 0, s.S, lam, s.J, lam) * clebschGordan(s1, l1, s2, -l2, s.S, lam);
			const double cgI =
			    clebschGordan(s.isobarL, 0, s.isobarS, 0, s.isobarJ, 0) * clebschGordan(0, 0, 0, 0, s.isobarS, 0);
			if (cgX == 0.0 || cgI == 0.0)
				continue;
			const double c = std::sqrt(s.L + 1.0) * cgX * std::sqrt(s.isobarL + 1.0) * cgI;
			LamTerm t{};
			t.lamIso = lamIso;
			t.plus0 = (int32_t)plan.dterms.size();
			wignerTerms(s.J, s.M, lam, plan.dterms);
			t.plus1 = (int32_t)plan.dterms.size();
			t.minus0 = t.minus1 = t.plus1;
			if (wMinus != 0.0) {
				wignerTerms(s.J, -s.M, lam, plan.dterms);
				t.minus1 = (int32_t)plan.dterms.size();
			}
			t.iso0 = (int32_t)plan.dterms.size();
			wignerTerms(s.isobarJ, lamIso, 0, plan.dterms);
			t.iso1 = (int32_t)plan.dterms.size();
			t.cPlus = c * wPlus;
			t.cMinus = c * wMinus;
			t.mPlus = s.M;
			t.mMinus = -s.M;
			plan.lams.push_back(t);
		}
		w.lam1 = (int32_t)plan.lams.size();
		plan.waves.push_back(w);
	}
	// isobar classes: waves whose mass dependence (kind and parameters) and
	// isobar barrier factor agree share their product per event and term
	auto sameIsobar = [](const WaveDev& x, const WaveDev& y) {
		if (x.massDep != y.massDep || x.LI != y.LI || x.a != y.a || x.b != y.b || x.m0 != y.m0 || x.g0 != y.g0 ||
		    x.q0 != y.q0 || x.f2q0 != y.f2q0 || x.ma != y.ma || x.mb != y.mb || x.q02 != y.q02)
			return false;
		for (int k = 0; k < 10; ++k)
			if (x.mdp[k] != y.mdp[k])
				return false;
		return true;
	};
	for (size_t i = 0; i < plan.waves.size(); ++i) {
		WaveDev& w = plan.waves[i];
		w.iso = (int32_t)i;
		for (size_t j = 0; j < i; ++j)
			if (sameIsobar(plan.waves[j], w)) {
				w.iso = plan.waves[j].iso;
				break;
			}
	}
	plan.order.resize(plan.waves.size());
	for (size_t i = 0; i < plan.order.size(); ++i)
		plan.order[i] = (int32_t)i;
	// waves of one topology class together (they share the kinematics), within
	// a class those of one mass dependence and isobar class, then of one X-vertex
	// L (they share the cached values)
	std::stable_sort(plan.order.begin(), plan.order.end(), [&](int32_t x, int32_t y) {
		const WaveDev &a = plan.waves[x], &b = plan.waves[y];
		if (a.topo != b.topo)
			return a.topo < b.topo;
		if (a.massDep != b.massDep)
			return a.massDep < b.massDep;
		if (a.iso != b.iso)
			return a.iso < b.iso;
		return a.LX < b.LX;
	});
	fillFp32Copies(plan);
	return std::string();
}

}  // namespace iso
}  // namespace pwa
