// isobar_math.cuh -- per-event arithmetic of the three-body isobar decay
// amplitudes in the helicity or canonical formalism, written once for the
// GPU kernel (isobar.cu): frames and kinematics in FP64, the per-wave part in
// FP64 or FP32 (template parameter).  The functions are plain C++ on POD
// views of the wave plan, so the same source also compiles as host code (the
// CPU tests compile it with g++ to check the arithmetic against the FP64
// oracle without a GPU).
//
// Reference: isobarHelicityAmplitude (decayAmplitude/isobarHelicityAmplitude.cc:
// 64-195), isobarCanonicalAmplitude (decayAmplitude/isobarCanonicalAmplitude.cc:
// 64-190), isobarAmplitude (decayAmplitude/isobarAmplitude.cc:98-330), mass
// dependences (decayAmplitude/massDependence.cc:169-862), barrier factors and
// Breit-Wigner (utilities/physUtils.hpp:75-300).
//
// Frames.  The reference reaches the Gottfried-Jackson frame by a rotation
// that puts beam x X on the y axis, a boost into the X rest frame and a
// rotation about y that puts the beam on z (isobarAmplitude.cc:137-171).
// The result is the orthonormal basis z = beam direction in the X rest
// frame, y = unit(beam x X) in the lab (a boost along X keeps the components
// perpendicular to X), x = y x z; here the final-state momenta are boosted
// into the X rest frame and projected on that basis, once per event and
// once more per symmetrisation term that exchanges particles of different
// mass (the term keeps each slot's mass, so X changes).  The isobar's
// helicity frame (isobarHelicityAmplitude.cc:64-84) is likewise the basis
// z = isobar direction, y = unit(z_GJ x isobar), x = y x z followed by a boost
// along z.  In the measure-zero case of an isobar along z_GJ (y undefined)
// the kernel takes y = y_GJ.  The canonical formalism
// (decayAmplitude/isobarCanonicalAmplitude.cc:64-190) reaches the isobar's
// rest frame by the boost alone, keeping the Gottfried-Jackson axes.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define PWA_HD __host__ __device__ __forceinline__
#else
#define PWA_HD inline
#endif

namespace pwa {
namespace iso {

constexpr int kMaxSpin = 16;      // 2J: spins up to 8
constexpr int kMaxL = 14;         // 2L: barrier factors up to L = 7
constexpr int kMaxPerms = 6;      // Bose terms of three particles
constexpr double kPr = 0.1973;    // GeV/c, 1 fm interaction radius

enum {
	kMassFlat = 0,
	kMassRelBw = 1,
	kMassConstBw = 2,
	kMassRhoBw = 3,
	kMassF0980Bw = 4,
	kMassF0980Flatte = 5,
	kMassPiPiSM = 6,        // pi pi S-wave, Au-Morgan-Pennington M solution
	kMassPiPiSVes = 7,      // ... VES sheet with the f0(980) subtracted
	kMassPiPiSKachaev = 8,  // ... Kachaev's reduced parameter set
	kMassBinned = 9,        // 1 inside a mass bin [m0, g0), else 0
	kMassRhoPrime = 10,     // (4 BW(rho(1450)) - 3 BW(rho(1700))) / 7
	kMassKPiSGlass = 11,    // K pi S-wave, LASS form (parameters per wave)
	kMassKPiSPalano = 12    // K pi S-wave, Palano-Pennington K-matrix
};
constexpr double kMassEta = 0.547862;

// f0(980) Flatte form with the BES II parameters (massDependence.cc:395-445)
// and the charged pion and kaon masses of the particle table
constexpr double kFlatteM0 = 0.965, kFlatteG1 = 0.165, kFlatteG2G1 = 4.21;
constexpr double kMassPiCharged = 0.13957039, kMassKCharged = 0.493677;
constexpr double kMassPiNeutral = 0.1349768, kMassKNeutral = 0.497611;

// Au, Morgan, Pennington, Phys. Rev. D 35 (1987) 1633, Table 1, M solution
// (the parameters of massDependence.cc:449-500).  The amplitude is T_00 of
// (M - i rho)^-1 with M's off-diagonal elements set to zero, so only the
// (0, 0) elements enter: residues of the poles at s_0, s_1 and the
// background polynomial in (s / 4 m_K^2 - 1).
constexpr double kAmpA0 = 0.1131, kAmpF1 = 0.1968;
constexpr double kAmpS0 = -0.0074, kAmpS1 = 0.9828;
constexpr double kAmpC0 = 0.0337, kAmpC1 = -0.3185, kAmpC2 = -0.0942, kAmpC3 = -0.5927, kAmpC4 = 0.1957;
// VES: f0(980) Breit-Wigner subtracted with this coupling (massDependence.cc:578-604)
constexpr double kVesF0Mass = 0.9837, kVesF0Width = 0.0376, kVesCouplingRe = -0.3743, kVesCouplingIm = 0.3197;

// d^j_{m n}(theta) = sum over terms of coef * cos(theta/2)^a * sin(theta/2)^b
struct DTerm {
	double coef;
	int32_t a, b;
	float coefF;                    // coef in FP32 (complex64 mode)
	int32_t pad;
};

// one spin projection of the isobar in one wave: the X-vertex angular part
// cPlus e^{i mPlus phi/2} dPlus(theta) + cMinus e^{i mMinus phi/2} dMinus(theta)
// (couplings, norms and the reflectivity combination folded into cPlus,
// cMinus) times the isobar vertex e^{i lamIso phiH/2} dIso(thetaH).
// Helicity formalism: mPlus/mMinus = +-M, dPlus/dMinus = d^J_{+-M lam},
// dIso = d^j_{lam 0}.  Canonical formalism: mPlus/mMinus = +-M - m,
// dPlus/dMinus = d^L_{+-M-m, 0} (spherical harmonics Y_L), dIso = d^l_{m 0}.
struct LamTerm {
	int32_t lamIso;                 // 2 lambda (helicity) or 2 m (canonical) of the isobar
	int32_t plus0, plus1;           // DTerm range of dPlus
	int32_t minus0, minus1;         // DTerm range of dMinus (empty if unused)
	int32_t iso0, iso1;             // DTerm range of dIso
	int32_t mPlus, mMinus;          // phase multipliers (units of 1/2)
	double cPlus, cMinus;
	float cPlusF, cMinusF;          // FP32 copies (complex64 mode)
};

struct WaveDev {
	int32_t a, b, c;                // isobar daughters 1, 2 and the bachelor (final-state slots)
	int32_t bachelorFirst;          // X-vertex daughter 1 (the analyser) is the bachelor
	int32_t M;                      // 2M of X
	int32_t LX, LI;                 // 2L of the X and isobar vertices (barrier factors)
	int32_t massDep;
	double m0, g0;                  // isobar mass and width (binned: the bin's lower and upper edge)
	double q0, f2q0;                // breakup momentum at m0 and F_L^2(q0) (relativistic BW)
	double ma, mb;                  // isobar daughter masses
	double q02;                     // breakup momentum squared at m0 (rho BW)
	double mdp[10];                 // parameters of the K pi S-wave forms
	int32_t lam0, lam1;             // LamTerm range
	int32_t term0, term1;           // SymTerm range (symmetrisation terms)
	int32_t topo;                   // topology class (waves of one class share kinematics)
	int32_t iso;                    // isobar class: waves of equal mass dependence and isobar L
	int32_t q0Zero;                 // q0 == 0 (the relativistic Breit-Wigner is then 0)
	// FP32 copies for the complex64 mode, whose per-wave arithmetic must not
	// convert FP64 constants (a conversion runs on the FP64 pipe)
	float m0F, g0F, q0F, f2q0F, maF, mbF, q02F;
	float dmHi, dmLo;               // the mass M that M^2 - m^2 is formed with (m0; Flatte: its M0), hi + lo
};

// one symmetrisation term of a wave: final-state permutation (index into the
// six permutations of three slots) and its factor (Bose times isospin)
struct SymTerm {
	int32_t perm;
	float factorF;                  // factor in FP32 (complex64 mode)
	double factor;
};

// read-only view of a wave plan (device or host pointers)
struct PlanView {
	const WaveDev* waves;
	const int32_t* order;           // waves sorted by topology class
	const LamTerm* lams;
	const DTerm* dterms;
	const double* bfPoly;           // [8][8]: P_l(z) coefficients of z^0..z^l
	const double* bfNorm;           // [8]: P_l(1)
	const float* bfPolyF;           // FP32 copies (complex64 mode)
	const float* bfNormF;
	const int32_t* perms;           // [6][3]: the permutations of three slots; slot i takes particle perms[p][i]
	const SymTerm* terms;
	uint32_t nWaves, pad0;
	double masses[3], beamMass;
	int32_t spaceInversion, reflection;
	int32_t canonical;              // isobar rest frame by a boost alone (canonical formalism)
	int32_t pad;
};

template <typename T>
struct C2T {
	T re, im;
};
typedef C2T<double> C2;
template <typename T>
PWA_HD C2T<T> cmul(C2T<T> x, C2T<T> y)
{
	return C2T<T>{x.re * y.re - x.im * y.im, x.re * y.im + x.im * y.re};
}
template <typename T>
PWA_HD C2T<T> cadd(C2T<T> x, C2T<T> y)
{
	return C2T<T>{x.re + y.re, x.im + y.im};
}
template <typename T>
PWA_HD C2T<T> cscale(C2T<T> x, T s)
{
	return C2T<T>{x.re * s, x.im * s};
}
PWA_HD C2T<double> cexpi(double x)
{
#if defined(__CUDA_ARCH__)
	double s, c;
	sincos(x, &s, &c);
	return C2T<double>{c, s};
#else
	return C2T<double>{std::cos(x), std::sin(x)};
#endif
}
PWA_HD C2T<float> cexpi(float x)
{
#if defined(__CUDA_ARCH__)
	float s, c;
	sincosf(x, &s, &c);
	return C2T<float>{c, s};
#else
	return C2T<float>{std::cos(x), std::sin(x)};
#endif
}

// a plan constant in the arithmetic type T: the FP64 value or its FP32 copy
template <typename T>
PWA_HD T pick(double d, float f);
template <>
PWA_HD double pick<double>(double d, float) { return d; }
template <>
PWA_HD float pick<float>(double, float f) { return f; }

struct V3 {
	double x, y, z;
};
PWA_HD V3 vadd(V3 u, V3 v) { return V3{u.x + v.x, u.y + v.y, u.z + v.z}; }
PWA_HD V3 vscale(V3 u, double s) { return V3{u.x * s, u.y * s, u.z * s}; }
PWA_HD double vdot(V3 u, V3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
PWA_HD V3 vcross(V3 u, V3 v) { return V3{u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x}; }
PWA_HD V3 vunit(V3 u)
{
	const double n = sqrt(vdot(u, u));
	return n > 0 ? vscale(u, 1.0 / n) : u;
}

struct LV {
	V3 p;
	double e;
};

// (e, p) in the rest frame of (eX, pX) of mass mX:
// e' = (e eX - p.pX) / mX,  p' = p - pX (e + e') / (eX + mX)
PWA_HD LV toRest(LV v, V3 pX, double eX, double mX)
{
	const double e1 = (v.e * eX - vdot(v.p, pX)) / mX;
	return LV{vadd(v.p, vscale(pX, -(v.e + e1) / (eX + mX))), e1};
}

template <typename T>
PWA_HD T ipow(T x, int n)
{
	T r = T(1);
	while (n > 0) {
		if (n & 1)
			r *= x;
		x *= x;
		n >>= 1;
	}
	return r;
}

template <typename T>
PWA_HD T dEval(const DTerm* t, int t0, int t1, T c, T s)
{
	T d = T(0);
	for (int k = t0; k < t1; ++k)
		d += pick<T>(t[k].coef, t[k].coefF) * ipow(c, t[k].a) * ipow(s, t[k].b);
	return d;
}

// the barrier polynomials' coefficients in T (the FP32 copies exist only in
// plans built for the kernel; the FP64 path reads only the FP64 arrays)
template <typename T>
PWA_HD T bfPolyAt(const PlanView& P, int i);
template <>
PWA_HD double bfPolyAt<double>(const PlanView& P, int i) { return P.bfPoly[i]; }
template <>
PWA_HD float bfPolyAt<float>(const PlanView& P, int i) { return P.bfPolyF[i]; }
template <typename T>
PWA_HD T bfNormAt(const PlanView& P, int l);
template <>
PWA_HD double bfNormAt<double>(const PlanView& P, int l) { return P.bfNorm[l]; }
template <>
PWA_HD float bfNormAt<float>(const PlanView& P, int l) { return P.bfNormF[l]; }

// Blatt-Weisskopf F_L(q)^2 = P_l(1) z^l / P_l(z), z = (q / 0.1973)^2, L = 2l
template <typename T>
PWA_HD T barrierF2(const PlanView& P, int L, T q)
{
	const int l = L / 2;
	if (l == 0)
		return T(1);
	const T z = (q * q) / T(kPr * kPr);
	T den = bfPolyAt<T>(P, 8 * l + l);
	for (int k = l - 1; k >= 0; --k)
		den = den * z + bfPolyAt<T>(P, 8 * l + k);
	return bfNormAt<T>(P, l) * ipow(z, l) / den;
}

template <typename T>
PWA_HD T breakup2(T M, T m1, T m2)
{
	const T s = m1 + m2, d = m1 - m2;
	return (M - s) * (M + s) * (M - d) * (M + d) / (T(4) * M * M);
}

// 2 k / m with the complex breakup momentum k of two particles of mass m1
// (imaginary below threshold, physUtils.hpp:108-120)
PWA_HD C2T<double> rhoOf(double m, double m1)
{
	const double q2 = breakup2<double>(m, m1, m1);
	const double r = 2.0 * sqrt(q2 < 0 ? -q2 : q2) / m;
	return q2 < 0 ? C2T<double>{0.0, r} : C2T<double>{r, 0.0};
}

// KPiSGLASS::amp (massDependence.cc:700-722): LASS-type K pi S-wave,
// p = a, r, M0, G0, phiF, phiR, phiRsin, F, R, MMax; atan as in the reference
PWA_HD C2T<double> kPiSGlass(double M, const double* p)
{
	const double mk = kMassKCharged, mpi = kMassPiCharged;
	if (!(M > mk + mpi && M < p[9]))
		return C2T<double>{0.0, 0.0};
	const double q = sqrt(breakup2<double>(M, mk, mpi));
	const double q0 = sqrt(fabs(breakup2<double>(p[2], mk, mpi)));
	const double G = p[3] * p[2] / M * q / q0;
	const double dR = atan(p[2] * G / (p[2] * p[2] - M * M));
	const double dF = atan(2.0 * p[0] * q / (2.0 + p[0] * p[1] * q * q));
	const double aF = dF + p[4];
	const double sF = p[7] * sin(aF), sR = p[8] * sin(dR + p[6]);
	// F sin(aF) e^{i aF} + R sin(dR + phiRsin) e^{i (dR + phiR + 2 aF)}
	const double ph = dR + p[5] + 2.0 * aF;
	const double scale = 0.5 * M / q;
	return C2T<double>{scale * (sF * cos(aF) + sR * cos(ph)), scale * (sF * sin(aF) + sR * sin(ph))};
}

// KPiSPalanoPennington::amp (massDependence.cc:770-828): two-channel (K pi,
// K eta) K-matrix with an Adler zero, published parameters; T_11
PWA_HD C2T<double> kPiSPalano(double M, double MMax)
{
	const double mk = kMassKCharged, mpi = kMassPiCharged;
	if (!(M > mk + mpi && M < MMax))
		return C2T<double>{0.0, 0.0};
	const double sTop = 5.832, sBot = 0.36, sa = 1.7991, sb = 8.3627;
	const double ga0 = 0.3139, ga1 = -0.00775, gb0 = 1.1804, gb1 = -0.22335;
	const double sKpi = mk * mk + mpi * mpi, sA = 0.87753 * sKpi;
	const double s = M * M, x = (2.0 * s - (sTop + sBot)) / (sTop - sBot);
	const double pre = (s - sA) / sKpi;
	auto poly = [x](double c0, double c1, double c2, double c3) { return c0 + x * (c1 + x * (c2 + x * c3)); };
	const double K11 = pre * (ga0 * ga0 / (sa - s) + gb0 * gb0 / (sb - s) + poly(-0.1553, 0.0909, 0.8618, 0.0629));
	const double K12 = pre * (ga0 * ga1 / (sa - s) + gb0 * gb1 / (sb - s) + poly(0.0738, 0.3866, 1.2195, 0.8390));
	const double K22 = pre * (ga1 * ga1 / (sa - s) + gb1 * gb1 / (sb - s) + poly(-0.0036, 0.2590, 1.6950, 2.2300));
	// rho = 2 q / M with complex breakup momenta (imaginary below threshold)
	auto rho = [M](double m1, double m2) {
		const double q2 = breakup2<double>(M, m1, m2);
		const double r = 2.0 * sqrt(q2 < 0 ? -q2 : q2) / M;
		return q2 < 0 ? C2T<double>{0.0, r} : C2T<double>{r, 0.0};
	};
	const C2T<double> r1 = rho(mk, mpi), r2 = rho(mk, kMassEta);
	const double detK = K11 * K22 - K12 * K12;
	// delta = 1 - i r1 K11 - i r2 K22 - r1 r2 detK;  T11 = (K11 - i r2 detK) / delta
	const C2T<double> r1r2 = cmul(r1, r2);
	const C2T<double> delta{1.0 + r1.im * K11 + r2.im * K22 - r1r2.re * detK,
	                        -r1.re * K11 - r2.re * K22 - r1r2.im * detK};
	const C2T<double> num{K11 + r2.im * detK, -r2.re * detK};
	const double n2 = delta.re * delta.re + delta.im * delta.im;
	return C2T<double>{(num.re * delta.re + num.im * delta.im) / n2, (num.im * delta.re - num.re * delta.im) / n2};
}

// piPiSWaveAuMorganPennington{M,Ves,Kachaev}::amp (massDependence.cc:505-625),
// FP64 (the poles cancel near s_1)
PWA_HD C2T<double> piPiSWave(double m, int variant)
{
	double s = m * m;
	if (fabs(s - kAmpS1) < 1e-6) {
		m += 1e-6;
		s = m * m;
	}
	C2T<double> rho;
	if (variant == kMassPiPiSVes) {
		rho = rhoOf(m, kMassPiCharged);
	} else {
		const C2T<double> rc = rhoOf(m, kMassPiCharged), rn = rhoOf(m, kMassPiNeutral);
		rho = C2T<double>{0.5 * (rc.re + rn.re), 0.5 * (rc.im + rn.im)};
	}
	const double mk = 0.5 * (kMassKCharged + kMassKNeutral);
	const double scale = s / (4.0 * mk * mk) - 1.0;
	const bool kachaev = variant == kMassPiPiSKachaev;
	double M = kAmpA0 / (s - kAmpS0) + (kachaev ? 0.0 : kAmpF1 * kAmpF1 / (s - kAmpS1));
	const double x = scale, x2 = x * x;
	M += kAmpC0 + kAmpC1 * x + kAmpC2 * x2 + kAmpC3 * x2 * x + (kachaev ? 0.0 : kAmpC4 * x2 * x2);
	// 1 / (M - i rho) = 1 / ((M + Im rho) - i Re rho)
	const double dRe = M + rho.im, dIm = -rho.re, n2 = dRe * dRe + dIm * dIm;
	C2T<double> amp{dRe / n2, -dIm / n2};
	if (variant == kMassPiPiSVes && m > 2.0 * kMassPiCharged) {
		const double q = sqrt(breakup2<double>(m, kMassPiCharged, kMassPiCharged));
		const double q0 = sqrt(breakup2<double>(kVesF0Mass, kMassPiCharged, kMassPiCharged));
		const double C = kVesF0Mass * kVesF0Width * (q / q0);
		const double A = C * (m / q), B = kVesF0Mass * kVesF0Mass - m * m;
		const double f = A / (B * B + C * C);
		const C2T<double> bw{f * B, f * C};
		amp.re -= kVesCouplingRe * bw.re - kVesCouplingIm * bw.im;
		amp.im -= kVesCouplingRe * bw.im + kVesCouplingIm * bw.re;
	}
	return amp;
}

// dm2 = m0^2 - mI^2 is formed in FP64 (it cancels near the peak, where FP32
// would lose a narrow width's resolution); mId is the FP64 isobar mass for
// the breakup momenta of the Flatte form, which cancel at the K K threshold
template <typename T>
PWA_HD C2T<T> massDependence(const PlanView& P, const WaveDev& w, T mI, T dm2, double mId)
{
	const T m0 = pick<T>(w.m0, w.m0F), g0 = pick<T>(w.g0, w.g0F);
	const T ma = pick<T>(w.ma, w.maF), mb = pick<T>(w.mb, w.mbF), q0 = pick<T>(w.q0, w.q0F);
	if (w.massDep == kMassRelBw) {
		if (w.q0Zero)
			return C2T<T>{T(0), T(0)};
		const T q2 = breakup2<T>(mI, ma, mb);
		const T q = q2 > T(0) ? sqrt(q2) : T(0);
		const T G = g0 * (m0 / mI) * (q / q0) * (barrierF2<T>(P, w.LI, q) / pick<T>(w.f2q0, w.f2q0F));
		const T A = m0 * g0, B = dm2, Cc = m0 * G;
		const T f = A / (B * B + Cc * Cc);
		return C2T<T>{f * B, f * Cc};
	}
	if (w.massDep == kMassConstBw) {
		const T A = m0 * g0, B = dm2;
		const T f = A / (B * B + A * A);
		return C2T<T>{f * B, f * A};
	}
	if (w.massDep == kMassRhoBw) {
		// rhoBreitWigner (massDependence.cc:324-359): F = 2 q^2 / (q0^2 + q^2)
		const T q2r = breakup2<T>(mI, ma, mb);
		const T q2 = q2r > T(0) ? q2r : T(0);
		const T q02 = pick<T>(w.q02, w.q02F);
		const T F = T(2) * q2 / (q02 + q2);
		const T G = g0 * (m0 / mI) * (sqrt(q2) / q0) * F;
		const T A = m0 * g0 * sqrt(F), B = dm2, Cc = m0 * G;
		const T f = A / (B * B + Cc * Cc);
		return C2T<T>{f * B, f * Cc};
	}
	if (w.massDep == kMassF0980Bw) {
		// f0980BreitWigner (massDependence.cc:363-390): Gamma = Gamma0 q / q0;
		// at q = 0 (an isobar exactly at its threshold) 0/0 as in the reference
		const T q2 = breakup2<T>(mI, ma, mb);
		const T q = q2 > T(0) ? sqrt(q2) : T(0);
		const T Cc = m0 * g0 * (q / q0);
		const T A = Cc * mI / q, B = dm2;
		const T f = A / (B * B + Cc * Cc);
		return C2T<T>{f * B, f * Cc};
	}
	if (w.massDep == kMassF0980Flatte) {
		// 1 / (M0^2 - m^2 - i g1 (rho_pipi + g2/g1 rho_KK)), rho = 2 k / m with
		// the complex breakup momenta k (imaginary below threshold)
		const T kPi2 = T(breakup2<double>(mId, kMassPiCharged, kMassPiCharged));
		const T kK2 = T(breakup2<double>(mId, kMassKCharged, kMassKCharged));
		const T rPi = T(2) * sqrt(kPi2 < T(0) ? -kPi2 : kPi2) / mI;
		const T rK = T(2) * sqrt(kK2 < T(0) ? -kK2 : kK2) / mI;
		const T reRho = (kPi2 < T(0) ? T(0) : rPi) + T(kFlatteG2G1) * (kK2 < T(0) ? T(0) : rK);
		const T imRho = (kPi2 < T(0) ? rPi : T(0)) + T(kFlatteG2G1) * (kK2 < T(0) ? rK : T(0));
		// denominator d = (M0^2 - m^2 + g1 Im rho) - i g1 Re rho; 1/d = conj(d) / |d|^2
		const T dRe = dm2 + T(kFlatteG1) * imRho;
		const T dIm = -T(kFlatteG1) * reRho;
		const T n2 = dRe * dRe + dIm * dIm;
		return C2T<T>{dRe / n2, -dIm / n2};
	}
	if (w.massDep == kMassRhoPrime) {
		// rhoPrimeMassDep (massDependence.cc:830-862): constant-width Breit-Wigners
		// of rho(1450) (1.465, 0.235) and rho(1700) (1.700, 0.220) mixed 4 : -3
		const double m2 = mId * mId;
		const double A1 = 1.465 * 0.235, B1 = 1.465 * 1.465 - m2, f1 = A1 / (B1 * B1 + A1 * A1);
		const double A2 = 1.700 * 0.220, B2 = 1.700 * 1.700 - m2, f2 = A2 / (B2 * B2 + A2 * A2);
		return C2T<T>{T((4.0 * f1 * B1 - 3.0 * f2 * B2) / 7.0), T((4.0 * f1 * A1 - 3.0 * f2 * A2) / 7.0)};
	}
	if (w.massDep == kMassKPiSGlass || w.massDep == kMassKPiSPalano) {
		const C2T<double> a = w.massDep == kMassKPiSGlass ? kPiSGlass(mId, w.mdp)
		                                                  : kPiSPalano(mId, w.mdp[0] > 0 ? w.mdp[0] : 2.4);
		return C2T<T>{T(a.re), T(a.im)};
	}
	if (w.massDep == kMassBinned)  // binnedMassDependence (massDependence.cc:212-230), FP64 mass
		return C2T<T>{(mId >= w.m0 && mId < w.g0) ? T(1) : T(0), T(0)};
	if (w.massDep >= kMassPiPiSM && w.massDep <= kMassPiPiSKachaev) {
		const C2T<double> a = piPiSWave(mId, w.massDep);
		return C2T<T>{T(a.re), T(a.im)};
	}
	return C2T<T>{T(1), T(0)};
}

// kinematics of one symmetrisation term for one topology class, in the
// arithmetic type T of the per-wave part
template <typename T>
struct Kin {
	// analyser of the X vertex in the GJ frame: e^{i phi/2}, cos/sin(theta/2)
	// and their squares, |p|
	C2T<T> u;
	T cX, sX, c2X, s2X, qX;
	// isobar daughter 1 in the isobar's helicity (canonical: rest) frame
	C2T<T> uH;
	T cI, sI, c2I, s2I, qI;
	T mI, mIlo;                     // isobar mass in T; FP32: mI + mIlo is the FP64 mass to ~2^-48
	double mId;                     // isobar mass in FP64
	// values shared by the waves of this kinematics, cached on first use:
	// the mass dependence of the isobar mass alone (by mass-dependence kind),
	// mass dependence x sqrt(F_LI(qI)) (by isobar class), sqrt(F_LX(qX)) (by LX)
	int32_t mdKind, isoKey, lxKey;
	C2T<T> md, isoVal;
	T lxVal;
	PWA_HD void clearCaches()
	{
		mdKind = isoKey = lxKey = -1;
	}
};

// mass dependences that depend on the isobar mass alone (no per-wave
// parameters): evaluated once per topology class and symmetrisation term
PWA_HD bool massDepOfMassAlone(int k)
{
	return k == kMassF0980Flatte || k == kMassRhoPrime || (k >= kMassPiPiSM && k <= kMassPiPiSKachaev);
}

PWA_HD double phiOf(double x, double y) { return (x == 0.0 && y == 0.0) ? 0.0 : atan2(y, x); }

PWA_HD void halfAngle(double perp, double z, double* c, double* s)
{
	const double th = (perp == 0.0 && z == 0.0) ? 0.0 : atan2(perp, z);
#if defined(__CUDA_ARCH__)
	sincos(0.5 * th, s, c);
#else
	*s = std::sin(0.5 * th);
	*c = std::cos(0.5 * th);
#endif
}

// angles from FP64 components, evaluated in FP32 (the complex64 mode: the
// per-wave arithmetic that consumes them is FP32)
PWA_HD float phiOfF(double x, double y)
{
	const float xf = (float)x, yf = (float)y;
	return (xf == 0.f && yf == 0.f) ? 0.f : atan2f(yf, xf);
}

PWA_HD void halfAngleF(double x, double y, double z, float* c, float* s, float* q)
{
	const float xf = (float)x, yf = (float)y, zf = (float)z;
	const float perp = sqrtf(xf * xf + yf * yf);
	const float th = (perp == 0.f && zf == 0.f) ? 0.f : atan2f(perp, zf);
	float sf, cf;
#if defined(__CUDA_ARCH__)
	sincosf(0.5f * th, &sf, &cf);
#else
	sf = std::sin(0.5f * th);
	cf = std::cos(0.5f * th);
#endif
	*s = sf;
	*c = cf;
	*q = sqrtf(perp * perp + zf * zf);
}

// g: the Gottfried-Jackson four-vectors of the final-state slots of one
// symmetrisation term.  T = double: FP64 throughout.  T = float (complex64
// amplitudes): the boosts, the isobar mass and momentum and the helicity
// frame's boost along z stay in FP64 (they cancel); the angles and
// magnitudes the per-wave FP32 arithmetic consumes are computed in FP32
// from the FP64 components, which keeps GB300's narrow FP64 pipe off the
// transcendental functions.
template <typename T>
PWA_HD Kin<T> kinematics(const LV g[3], const WaveDev& w, bool canonical);

template <>
PWA_HD Kin<float> kinematics<float>(const LV g[3], const WaveDev& w, bool canonical)
{
	const LV A = g[w.a], B = g[w.b], Cb = g[w.c];
	const LV I{vadd(A.p, B.p), A.e + B.e};
	Kin<float> k;
	k.clearCaches();
	const V3 d1 = w.bachelorFirst ? Cb.p : I.p;
	k.u = cexpi(0.5f * phiOfF(d1.x, d1.y));
	halfAngleF(d1.x, d1.y, d1.z, &k.cX, &k.sX, &k.qX);
	k.c2X = k.cX * k.cX;
	k.s2X = k.sX * k.sX;
	const double pI = sqrt(vdot(I.p, I.p));
	k.mId = sqrt((I.e - pI) * (I.e + pI));
	k.mI = (float)k.mId;
	k.mIlo = (float)(k.mId - (double)k.mI);
	double ax, ay, az;
	if (canonical) {
		const LV r = toRest(A, I.p, I.e, k.mId);
		ax = r.p.x;
		ay = r.p.y;
		az = r.p.z;
	} else {
		// helicity frame: transverse axes in FP32, the boost along z in FP64
		const float ix = (float)I.p.x, iy = (float)I.p.y, iz = (float)I.p.z;
		const float perpI = sqrtf(ix * ix + iy * iy), pIf = (float)pI;
		float yx = 0.f, yy = 1.f;
		if (perpI > 0.f) {
			yx = -iy / perpI;
			yy = ix / perpI;
		}
		// x = y cross z with z = I / |I|
		const float zx = ix / pIf, zy = iy / pIf, zz = iz / pIf;
		const float xx = yy * zz, xy = -yx * zz, xz = yx * zy - yy * zx;
		const float axf = (float)A.p.x, ayf = (float)A.p.y, azf = (float)A.p.z;
		ax = axf * xx + ayf * xy + azf * xz;
		ay = axf * yx + ayf * yy;
		az = (I.e * (vdot(A.p, I.p) / pI) - pI * A.e) / k.mId;
	}
	k.uH = cexpi(0.5f * phiOfF(ax, ay));
	halfAngleF(ax, ay, az, &k.cI, &k.sI, &k.qI);
	k.c2I = k.cI * k.cI;
	k.s2I = k.sI * k.sI;
	return k;
}

template <>
PWA_HD Kin<double> kinematics<double>(const LV g[3], const WaveDev& w, bool canonical)
{
	const LV A = g[w.a], B = g[w.b], Cb = g[w.c];
	const LV I{vadd(A.p, B.p), A.e + B.e};
	Kin<double> k;
	k.clearCaches();
	const V3 d1 = w.bachelorFirst ? Cb.p : I.p;
	const double perp1 = sqrt(d1.x * d1.x + d1.y * d1.y);
	k.u = cexpi(0.5 * phiOf(d1.x, d1.y));
	halfAngle(perp1, d1.z, &k.cX, &k.sX);
	k.c2X = k.cX * k.cX;
	k.s2X = k.sX * k.sX;
	k.qX = sqrt(vdot(d1, d1));
	const double pI = sqrt(vdot(I.p, I.p));
	k.mId = k.mI = sqrt((I.e - pI) * (I.e + pI));
	k.mIlo = 0.0;
	double ax, ay, az;
	if (canonical) {
		// rest frame of the isobar with the Gottfried-Jackson axes
		// (isobarCanonicalAmplitude.cc:94-108)
		const LV r = toRest(A, I.p, I.e, k.mI);
		ax = r.p.x;
		ay = r.p.y;
		az = r.p.z;
	} else {
		// helicity frame of the isobar
		const V3 zh = vunit(I.p);
		const double perpI = sqrt(I.p.x * I.p.x + I.p.y * I.p.y);
		const V3 yh = perpI > 0 ? V3{-I.p.y / perpI, I.p.x / perpI, 0.0} : V3{0.0, 1.0, 0.0};
		const V3 xh = vcross(yh, zh);
		ax = vdot(A.p, xh);
		ay = vdot(A.p, yh);
		az = (I.e * vdot(A.p, zh) - pI * A.e) / k.mI;
	}
	const double perpA = sqrt(ax * ax + ay * ay);
	k.uH = cexpi(0.5 * phiOf(ax, ay));
	halfAngle(perpA, az, &k.cI, &k.sI);
	k.c2I = k.cI * k.cI;
	k.s2I = k.sI * k.sI;
	k.qI = sqrt(perpA * perpA + az * az);
	return k;
}

// M^2 - mI^2 of a wave's Breit-Wigner denominator (M = m0; Flatte: its M0).
// It cancels near the peak, where a narrow width needs the resolution of
// the FP64 masses: FP64 for T = double; for T = float from the hi + lo FP32
// pairs of M and mI, whose difference of the hi parts is exact near the
// peak (Sterbenz), so the result carries FP32 relative accuracy.
PWA_HD double deltaM2(const WaveDev& w, const Kin<double>& k)
{
	const double m0 = w.massDep == kMassF0980Flatte ? kFlatteM0 : w.m0;
	return (m0 - k.mId) * (m0 + k.mId);
}
PWA_HD float deltaM2(const WaveDev& w, const Kin<float>& k)
{
	return ((w.dmHi - k.mI) + (w.dmLo - k.mIlo)) * (w.dmHi + k.mI);
}

// u^m for a unit complex u and an integer m of either sign (u^-1 = conj u),
// by repeated squaring
template <typename T>
PWA_HD C2T<T> cpowi(C2T<T> u, int m)
{
	if (m < 0) {
		u.im = -u.im;
		m = -m;
	}
	C2T<T> r{T(1), T(0)};
	while (m > 0) {
		if (m & 1)
			r = cmul(r, u);
		u = cmul(u, u);
		m >>= 1;
	}
	return r;
}

// d^j_{m n}(theta) from its Wigner terms t0..t1-1 (dEval's arguments): the
// power of cos(theta/2) falls and that of sin(theta/2) rises by 2 from one
// term to the next (wignerTerms), so the sum is c^a_last s^b_first times a
// homogeneous polynomial in c^2 and s^2, evaluated Horner-like
template <typename T>
PWA_HD T dHorner(const DTerm* t, int t0, int t1, T c, T s, T c2, T s2)
{
	if (t0 >= t1)
		return T(0);
	T r = pick<T>(t[t0].coef, t[t0].coefF), sk = T(1);
	for (int k = t0 + 1; k < t1; ++k) {
		sk *= s2;
		r = r * c2 + pick<T>(t[k].coef, t[k].coefF) * sk;
	}
	return r * ipow(c, t[t1 - 1].a) * ipow(s, t[t0].b);
}

// amplitude of wave w for one symmetrisation term; T is the arithmetic of
// the per-wave part.  k is the term's kinematics; the values that several
// waves share (mass dependence and isobar barrier factor of one isobar class,
// the X-vertex barrier factor of one L) are cached in it.
template <typename T>
PWA_HD C2T<T> termAmplitude(const PlanView& P, const WaveDev& w, Kin<T>& k)
{
	// e^{i lamIso phiH / 2} as a power of e^{i phiH / 2}, stepped by e^{i phiH}
	const C2T<T> stepH = cmul(k.uH, k.uH);
	C2T<T> eL{T(1), T(0)};
	C2T<T> sum{T(0), T(0)};
	// e^{i m phi / 2} of the X vertex, recomputed only when m changes
	// (helicity formalism: m = +-M for every isobar helicity of the wave)
	constexpr int kNone = 1 << 30;
	int mP = kNone, mM = kNone;
	C2T<T> eP{T(1), T(0)}, eM{T(1), T(0)};
	for (int t = w.lam0; t < w.lam1; ++t) {
		const LamTerm& L = P.lams[t];
		if (t == w.lam0)
			eL = cpowi(k.uH, L.lamIso);
		else
			for (int s = P.lams[t - 1].lamIso; s < L.lamIso; s += 2)
				eL = cmul(eL, stepH);
		C2T<T> x{T(0), T(0)};
		if (L.plus1 > L.plus0) {
			if (L.mPlus != mP) {
				mP = L.mPlus;
				eP = cpowi(k.u, mP);
			}
			x = cscale(eP, pick<T>(L.cPlus, L.cPlusF) * dHorner<T>(P.dterms, L.plus0, L.plus1, k.cX, k.sX, k.c2X, k.s2X));
		}
		if (L.minus1 > L.minus0) {
			if (L.mMinus != mM) {
				mM = L.mMinus;
				eM = (mP != kNone && mM == -mP) ? C2T<T>{eP.re, -eP.im} : cpowi(k.u, mM);
			}
			x = cadd(x, cscale(eM, pick<T>(L.cMinus, L.cMinusF) *
			                           dHorner<T>(P.dterms, L.minus0, L.minus1, k.cX, k.sX, k.c2X, k.s2X)));
		}
		const T dI = dHorner<T>(P.dterms, L.iso0, L.iso1, k.cI, k.sI, k.c2I, k.s2I);
		sum = cadd(sum, cmul(x, cscale(eL, dI)));
	}
	if (k.isoKey != w.iso) {
		C2T<T> md;
		if (massDepOfMassAlone(w.massDep)) {
			if (k.mdKind != w.massDep) {
				k.md = massDependence<T>(P, w, k.mI, deltaM2(w, k), k.mId);
				k.mdKind = w.massDep;
			}
			md = k.md;
		} else {
			md = massDependence<T>(P, w, k.mI, deltaM2(w, k), k.mId);
		}
		k.isoVal = cscale(md, static_cast<T>(sqrt(barrierF2<T>(P, w.LI, k.qI))));
		k.isoKey = w.iso;
	}
	if (k.lxKey != w.LX) {
		k.lxVal = static_cast<T>(sqrt(barrierF2<T>(P, w.LX, k.qX)));
		k.lxKey = w.LX;
	}
	return cscale(cmul(sum, k.isoVal), k.lxVal);
}

// Gottfried-Jackson four-vectors of the three final-state slots of one
// event and symmetrisation term: beam momentum bp, final-state momenta fp
// (lab); slot i takes the momentum of particle perm[i] and keeps its own
// mass (decayTopology::revertMomenta with particle::setMomentum), so X and
// the frame follow the permutation when it exchanges particles of different
// mass (isospin partners)
PWA_HD void gjFrame(const PlanView& P, const double bp[3], const double fp[3][3], const int32_t* perm, LV g[3])
{
	LV f[3];
	V3 pX{0.0, 0.0, 0.0};
	double eX = 0.0;
	for (int i = 0; i < 3; ++i) {
		const int k = perm[i];
		f[i].p = V3{fp[k][0], fp[k][1], fp[k][2]};
		f[i].e = sqrt(P.masses[i] * P.masses[i] + vdot(f[i].p, f[i].p));
		pX = vadd(pX, f[i].p);
		eX += f[i].e;
	}
	const double pXa = sqrt(vdot(pX, pX));
	const double mX = sqrt((eX - pXa) * (eX + pXa));
	const V3 b{bp[0], bp[1], bp[2]};
	const LV beam{b, sqrt(P.beamMass * P.beamMass + vdot(b, b))};
	const V3 z = vunit(toRest(beam, pX, eX, mX).p);
	const V3 y = vunit(vcross(b, pX));
	const V3 x = vcross(y, z);
	const double sgn = P.spaceInversion ? -1.0 : 1.0;
	const double sgnY = P.reflection ? -sgn : sgn;
	for (int i = 0; i < 3; ++i) {
		const LV r = toRest(f[i], pX, eX, mX);
		g[i] = LV{V3{sgn * vdot(r.p, x), sgnY * vdot(r.p, y), sgn * vdot(r.p, z)}, r.e};
	}
}

// all waves of one event; out is complex [wave][ld] as interleaved T
// (complex128 for T = double, complex64 for T = float: FP64 frames and
// kinematics, per-wave arithmetic in T)
template <typename T>
PWA_HD void eventAmplitudes(const PlanView& P, const double bp[3], const double fp[3][3], T* out, uint64_t ld,
                            uint64_t e)
{
	// the frame of the unpermuted event; a permutation that only exchanges
	// particles of equal mass (Bose terms) permutes its four-vectors
	LV g0[3];
	gjFrame(P, bp, fp, P.perms, g0);
	// kinematics per permutation, computed once per topology class on first use
	Kin<T> kin[kMaxPerms];
	uint32_t valid = 0;
	int topo = -1;
	for (uint32_t o = 0; o < P.nWaves; ++o) {
		const int wi = P.order[o];
		const WaveDev& w = P.waves[wi];
		if (w.topo != topo) {
			topo = w.topo;
			valid = 0;
		}
		C2T<T> a{T(0), T(0)};
		for (int t = w.term0; t < w.term1; ++t) {
			const SymTerm st = P.terms[t];
			if (!((valid >> st.perm) & 1u)) {
				const int32_t* perm = P.perms + 3 * st.perm;
				LV g[3];
				if (P.masses[perm[0]] == P.masses[0] && P.masses[perm[1]] == P.masses[1] &&
				    P.masses[perm[2]] == P.masses[2]) {
					for (int i = 0; i < 3; ++i)
						g[i] = g0[perm[i]];
				} else {
					gjFrame(P, bp, fp, perm, g);
				}
				kin[st.perm] = kinematics<T>(g, w, P.canonical != 0);
				valid |= 1u << st.perm;
			}
			a = cadd(a, cscale(termAmplitude<T>(P, w, kin[st.perm]), pick<T>(st.factor, st.factorF)));
		}
		out[2 * ((uint64_t)wi * ld + e)] = a.re;
		out[2 * ((uint64_t)wi * ld + e) + 1] = a.im;
	}
}

}  // namespace iso
}  // namespace pwa
