// isobar.cu -- GPU evaluation of the three-body isobar decay amplitudes
// (isobarHelicityAmplitude::amplitude, decayAmplitude/isobarAmplitude.cc:98-262,
// isobarHelicityAmplitude.cc:64-195).  One thread per event in a grid-stride
// loop: the thread reads its event's beam and final-state momenta (SoA rows,
// coalesced), builds the Gottfried-Jackson frame once, the kinematics of every
// symmetrisation term once per topology class, and writes one complex128
// amplitude per wave (row-major [wave][event], coalesced across the warp):
// complex128 with FP64 arithmetic throughout, or complex64 with the frames
// and kinematics in FP64 and the per-wave arithmetic in FP32 (GB300 runs FP32
// at many times its FP64 rate; the likelihood's amplitude store is complex64).
// The wave plan (couplings, D-function terms, barrier polynomials) is a few
// KB read by every thread through the read-only cache.
#include "isobar_math.cuh"
#include "pwa_internal.h"

#include <algorithm>

namespace pwa {

namespace {

constexpr int kIsoThreads = 128;
// eight blocks (32 warps) per SM: the per-event arithmetic is a long chain
// of dependent operations, and the kernel is latency-bound at the 12 warps
// its unconstrained register count allows (measured on 10^6 events x 88
// waves: 20.4 ms at 160 registers, 16.8 ms at 128, 10.9 ms at 64 with a
// few hundred bytes of spills to L1, 11.3 ms at 40, 12.5 ms at 32)
constexpr int kIsoBlocksPerSM = 8;

template <typename T>
__global__ void __launch_bounds__(kIsoThreads, kIsoBlocksPerSM) isobarAmplitudeKernel(iso::PlanView P, const double* __restrict__ beam,
                                                                     const double* __restrict__ fs, uint64_t n,
                                                                     T* __restrict__ amps)
{
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
		double bp[3], fp[3][3];
		for (int k = 0; k < 3; ++k)
			bp[k] = __ldg(beam + k * n + e);
		for (int i = 0; i < 3; ++i)
			for (int k = 0; k < 3; ++k)
				fp[i][k] = __ldg(fs + (uint64_t)(3 * i + k) * n + e);
		iso::eventAmplitudes<T>(P, bp, fp, amps, n, e);
	}
}

}  // namespace

int launchIsobarAmplitudes(const iso::PlanView& v, const double* beam, const double* fs, uint64_t n, void* amps,
                           bool fp32, cudaStream_t s)
{
	if (n == 0 || v.nWaves == 0)
		return kOk;
	int dev = 0, sms = 0;
	PWA_CHECK(cudaCheck(cudaGetDevice(&dev), "cudaGetDevice"));
	PWA_CHECK(cudaCheck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
	const uint64_t need = (n + kIsoThreads - 1) / kIsoThreads;
	const unsigned blocks = (unsigned)std::min<uint64_t>(need, (uint64_t)sms * kIsoBlocksPerSM * 2);
	if (fp32)
		isobarAmplitudeKernel<float><<<blocks, kIsoThreads, 0, s>>>(v, beam, fs, n, static_cast<float*>(amps));
	else
		isobarAmplitudeKernel<double><<<blocks, kIsoThreads, 0, s>>>(v, beam, fs, n, static_cast<double*>(amps));
	countLaunches(1);
	return cudaCheck(cudaGetLastError(), "isobar amplitude kernel");
}

}  // namespace pwa
