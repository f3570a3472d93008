// Test infrastructure: compiles the GPU kernel's per-event arithmetic
// (rootpwa_gb300/csrc/isobar_math.cuh) and the wave-plan builder as host
// code, so that the CPU tests check the arithmetic of the kernel against the
// FP64 oracle without a GPU.  Built by tests/test_isobar_host.py into a
// temporary directory; never part of the library.
#include "../rootpwa_gb300/csrc/isobar_plan.h"

// out: complex128 [wave][n] (fp32 = 0) or complex64 (fp32 = 1), as the kernel writes them
extern "C" int shim_amplitudes(const pwa_isobar_wave* waves, int nWaves, const double* masses, const int32_t* species,
                               double beamMass, int reflBasis, int bose, int spaceInversion, int reflection,
                               const double* beam, const double* fs, uint64_t n, void* out, int fp32,
                               int canonical, const int32_t* isospins /* [3][3]: 2I, 2I_3, P, or NULL */)
{
	pwa::iso::FsIsospin iso{};
	if (isospins)
		for (int i = 0; i < 3; ++i) {
			iso.I[i] = isospins[3 * i];
			iso.I3[i] = isospins[3 * i + 1];
			iso.P[i] = isospins[3 * i + 2];
		}
	std::vector<pwa_isobar_wave> ws(waves, waves + nWaves);
	for (const pwa_isobar_wave& w : ws)
		if (!pwa::iso::checkWave(w, reflBasis != 0).empty())
			return 1;
	pwa::iso::Plan plan;
	if (!pwa::iso::buildPlan(ws, masses, species, beamMass, reflBasis != 0, bose != 0, spaceInversion != 0,
	                         reflection != 0, canonical != 0, isospins ? &iso : nullptr, plan)
	         .empty())
		return 2;
	const pwa::iso::PlanView v = plan.view();
	for (uint64_t e = 0; e < n; ++e) {
		double bp[3], fp[3][3];
		for (int k = 0; k < 3; ++k)
			bp[k] = beam[k * n + e];
		for (int i = 0; i < 3; ++i)
			for (int k = 0; k < 3; ++k)
				fp[i][k] = fs[(3 * i + k) * n + e];
		if (fp32)
			pwa::iso::eventAmplitudes<float>(v, bp, fp, static_cast<float*>(out), n, e);
		else
			pwa::iso::eventAmplitudes<double>(v, bp, fp, static_cast<double*>(out), n, e);
	}
	return 0;
}
