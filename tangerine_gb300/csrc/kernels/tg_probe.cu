// FP32 issue-rate probe: the roofline denominator for the distance interpreter, which
// is bound by FP32 arithmetic issue rather than by HBM or the tensor cores.  Each thread
// runs eight independent fused multiply-add chains (fmaf is always fused), so the kernel
// issues one FFMA per lane per cycle when the SMs are saturated.
#include <cuda_runtime.h>

#include "tg_kernels.hpp"

namespace tg
{
	namespace
	{
		constexpr int kChains = 8;
		constexpr int kIters = 4096;

		__global__ void __launch_bounds__(256) Fp32PeakKernel(float seed, float* sink)
		{
			float a[kChains];
#pragma unroll
			for (int c = 0; c < kChains; ++c) a[c] = seed + (float)(threadIdx.x + c);
			const float m = 0.999999f, b = 1e-7f;
			for (int i = 0; i < kIters; ++i)
			{
#pragma unroll
				for (int c = 0; c < kChains; ++c) a[c] = fmaf(a[c], m, b);
			}
			float s = 0.0f;
#pragma unroll
			for (int c = 0; c < kChains; ++c) s += a[c];
			if (s == 12345.678f) sink[threadIdx.x] = s;   // keeps the chains live
		}
	}

	cudaError_t MeasureFp32Peak(double* tflops, cudaStream_t stream)
	{
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		float* sink = nullptr;
		cudaError_t e = cudaMalloc(&sink, 256 * sizeof(float));
		if (e != cudaSuccess) return e;
		cudaEvent_t t0, t1;
		cudaEventCreate(&t0);
		cudaEventCreate(&t1);
		const int blocks = sms * 8;
		Fp32PeakKernel<<<blocks, 256, 0, stream>>>(1.0f, sink);      // warm-up
		cudaEventRecord(t0, stream);
		const int reps = 10;
		for (int r = 0; r < reps; ++r) Fp32PeakKernel<<<blocks, 256, 0, stream>>>(1.0f, sink);
		cudaEventRecord(t1, stream);
		e = cudaEventSynchronize(t1);
		float ms = 0.0f;
		if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
		cudaEventDestroy(t0);
		cudaEventDestroy(t1);
		cudaFree(sink);
		if (e != cudaSuccess) return e;
		const double flops = 2.0 * kChains * (double)kIters * 256.0 * blocks * reps;
		*tflops = flops / (ms * 1e-3) / 1e12;
		return cudaGetLastError();
	}
}
