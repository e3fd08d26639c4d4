// Device self-checks:
// * the float evaluation of the smooth-blend term (BlendTermFloat in tg_sdfmath.hpp)
//   against the reference's double expression, over seeded inputs: realistic operand
//   ranges, values where m and the blend term cancel (the blended surface), operands at
//   scattered exponents, and arbitrary finite bit patterns;
// * the paired FP32 arithmetic of tg_pair.cuh against the scalar formulas, lane by lane:
//   single adds and multiplies on arbitrary finite bit patterns, a product followed by a
//   sum, the brush formulas and the affine transform on realistic points.
#include <cstdint>

#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_pair.cuh"

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

	namespace
	{
		__device__ __forceinline__ bool SameBits(float a, float b)
		{
			return __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
		}

		constexpr int kPairChecks = 9;

		__global__ void PairCheckKernel(uint64_t n, uint64_t seed, unsigned long long* counts)
		{
			unsigned long long bad[kPairChecks] = {};
			unsigned long long seen = 0;
			const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
			const PairUnits un = LoadPairUnits();
			for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
			{
				uint64_t z = Mix(seed ^ (i * 0xD1B54A32D192ED03ull));
				uint32_t u[12];
				for (int j = 0; j < 12; j += 2) { z = Mix(z); u[j] = (uint32_t)z; u[j + 1] = (uint32_t)(z >> 32); }
				++seen;
				// 0, 1: one add, one multiply on any finite bit patterns (subnormals included).
				const float a0 = Finite(u[0], 1.0f), a1 = Finite(u[1], -2.0f), b0 = Finite(u[2], 0.5f), b1 = Finite(u[3], 3.0f);
				const float2 s2 = Add2(make_float2(a0, a1), make_float2(b0, b1), un);
				if (!SameBits(s2.x, a0 + b0) || !SameBits(s2.y, a1 + b1)) ++bad[0];
				const float2 m2 = Mul2(make_float2(a0, a1), make_float2(b0, b1), un);
				if (!SameBits(m2.x, a0 * b0) || !SameBits(m2.y, a1 * b1)) ++bad[1];
				// 2: a product then a sum (never fused into one rounding).
				const float c0 = (Unit(u[4]) - 0.5f) * 4.0f, c1 = (Unit(u[5]) - 0.5f) * 4.0f;
				const float d0 = (Unit(u[6]) - 0.5f) * 4.0f, d1 = (Unit(u[7]) - 0.5f) * 4.0f;
				const float e0 = (Unit(u[8]) - 0.5f), e1 = (Unit(u[9]) - 0.5f);
				const float2 f2 = Add2(Mul2(make_float2(c0, c1), make_float2(d0, d1), un), make_float2(e0, e1), un);
				if (!SameBits(f2.x, c0 * d0 + e0) || !SameBits(f2.y, c1 * d1 + e1)) ++bad[2];
				// 3..7: brushes at points of [-2, 2]^3 with parameters in [0.1, 0.5].
				const float2 x = make_float2(c0, d0), y = make_float2(c1, d1), zz = make_float2(2.0f * e0 + 0.5f * e1, 4.0f * e1);
				const float p0 = 0.1f + 0.4f * Unit(u[10]), p1 = 0.1f + 0.4f * Unit(u[11]), p2 = 0.1f + 0.4f * Unit(u[4] ^ u[11]);
				const Vec3 q0(x.x, y.x, zz.x), q1(x.y, y.y, zz.y);
				float2 r = SdSphere2(x, y, zz, p0, un);
				if (!SameBits(r.x, SdSphere(q0, p0)) || !SameBits(r.y, SdSphere(q1, p0))) ++bad[3];
				r = SdBox2(x, y, zz, p0, p1, p2, un);
				if (!SameBits(r.x, SdBox(q0, Vec3(p0, p1, p2))) || !SameBits(r.y, SdBox(q1, Vec3(p0, p1, p2)))) ++bad[4];
				r = SdTorus2(x, y, zz, p0, p1 * 0.5f, un);
				if (!SameBits(r.x, SdTorus(q0, p0, p1 * 0.5f)) || !SameBits(r.y, SdTorus(q1, p0, p1 * 0.5f))) ++bad[5];
				r = SdCylinder2(x, y, zz, p0, p1, un);
				if (!SameBits(r.x, SdCylinder(q0, p0, p1)) || !SameBits(r.y, SdCylinder(q1, p0, p1))) ++bad[6];
				// 8: the affine transform (M * vec4(p, 1)).x = (m0*x + m1*y) + (m2*z + m3).
				const float4 M = make_float4(p0 - 0.3f, p1 - 0.3f, p2 - 0.3f, e0);
				const float2 t = AffineRow2(M, x, y, zz, un);
				if (!SameBits(t.x, (M.x * q0.x + M.y * q0.y) + (M.z * q0.z + M.w)) ||
					!SameBits(t.y, (M.x * q1.x + M.y * q1.y) + (M.z * q1.z + M.w))) ++bad[8];
				r = SdPlane2(x, y, zz, p0, p1, p2, un);
				if (!SameBits(r.x, SdPlane(q0, Vec3(p0, p1, p2))) || !SameBits(r.y, SdPlane(q1, Vec3(p0, p1, p2)))) ++bad[7];
			}
			atomicAdd(counts, seen);
			for (int c = 0; c < kPairChecks; ++c) atomicAdd(counts + 1 + c, bad[c]);
		}
	}

	cudaError_t LaunchPairCheck(uint64_t n, uint64_t seed, unsigned long long* counts, cudaStream_t stream)
	{
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		cudaError_t e = cudaMemsetAsync(counts, 0, (1 + kPairChecks) * sizeof(unsigned long long), stream);
		if (e != cudaSuccess) return e;
		PairCheckKernel<<<sms * 4, 256, 0, stream>>>(n, seed, counts);
		return cudaGetLastError();
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
