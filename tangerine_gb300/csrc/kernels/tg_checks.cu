// Device self-check of the float evaluation of the smooth-blend term
// (BlendTermFloat in tg_sdfmath.hpp) against the reference's double expression, over
// seeded inputs: realistic operand ranges, values where m and the blend term cancel (the
// blended surface), operands at scattered exponents, and arbitrary finite bit patterns.
#include <cstdint>

#include "tg_device.cuh"
#include "tg_kernels.hpp"

namespace tg
{
	namespace
	{
		__device__ __forceinline__ uint64_t Mix(uint64_t z)
		{
			z += 0x9E3779B97F4A7C15ull;
			z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
			z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
			return z ^ (z >> 31);
		}

		__device__ __forceinline__ float Unit(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

		__device__ __forceinline__ float Finite(uint32_t bits, float fallback)
		{
			const float f = __uint_as_float(bits);
			return isfinite(f) ? f : fallback;
		}

		__global__ void BlendCheckKernel(uint64_t n, uint64_t seed, unsigned long long* counts)
		{
			unsigned long long mismatches = 0, fallbacks = 0, checked = 0;
			const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
			for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
			{
				const uint64_t z0 = Mix(seed ^ (i * 0xD1B54A32D192ED03ull)), z1 = Mix(z0);
				const uint32_t u0 = (uint32_t)z0, u1 = (uint32_t)(z0 >> 32), u2 = (uint32_t)z1, u3 = (uint32_t)(z1 >> 32);
				float m, h, k;
				switch (u3 & 3u)
				{
				case 0:          // operands of the benchmark trees
					k = 0.001f + 0.2f * Unit(u0);
					h = k * Unit(u1);
					m = ((u2 & 1u) ? -1.0f : 1.0f) * exp2f(-24.0f + 26.0f * Unit(u2));
					break;
				case 1:          // m and the blend term nearly cancel
				{
					k = 0.001f + 0.5f * Unit(u0);
					h = k * (0.05f + 0.95f * Unit(u1));
					const float q = (h * h) * 0.25f / k;
					const float rel = ldexpf(Unit(u2) - 0.5f, -(int)((u3 >> 2) % 30u));
					m = q + q * rel;
					if (u3 & 0x80000000u) m = -m;
					break;
				}
				case 2:          // scattered exponents
					k = exp2f(-40.0f + 80.0f * Unit(u0));
					h = k * exp2f(-30.0f * Unit(u1));
					m = ((u2 & 1u) ? -1.0f : 1.0f) * exp2f(-60.0f + 120.0f * Unit(u2));
					break;
				default:         // any finite bit patterns (k positive)
					m = Finite(u0, 1.0f);
					h = Finite(u1, 0.5f);
					k = Finite(u2 & 0x7FFFFFFFu, 0.25f);
					break;
				}
				for (int sub = 0; sub < 2; ++sub)
				{
					float fast;
					if (BlendTermFloat(m, h * h, k, sub == 0, fast))
					{
						++checked;
						const float ref = BlendTermDouble(m, h, k, sub == 0);
						if (__float_as_uint(fast) != __float_as_uint(ref)) ++mismatches;
					}
					else ++fallbacks;
				}
			}
			atomicAdd(counts + 0, checked);
			atomicAdd(counts + 1, mismatches);
			atomicAdd(counts + 2, fallbacks);
		}
	}

	cudaError_t LaunchBlendCheck(uint64_t n, uint64_t seed, unsigned long long* counts, cudaStream_t stream)
	{
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		cudaError_t e = cudaMemsetAsync(counts, 0, 3 * sizeof(unsigned long long), stream);
		if (e != cudaSuccess) return e;
		BlendCheckKernel<<<sms * 8, 256, 0, stream>>>(n, seed, counts);
		return cudaGetLastError();
	}
}
