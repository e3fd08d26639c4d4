// Learned distance bound: hash-grid features and a 3 x 64 ReLU network, trained and
// evaluated with this file's own kernels.
//
// Encoding (multiresolution hash grid, Mueller et al. 2022, "Instant Neural Graphics
// Primitives", section 3): the domain box maps to the unit cube; level l has Res[l] cells
// per axis; each of a point's 8 cell corners indexes the level's table densely when the
// level's (Res + 1)^3 corners fit the table, else through the paper's spatial hash
// (x * 1) xor (y * 2654435761) xor (z * 805459861) mod TableSize; the trilinear blend of
// the corners' 2 features gives 2 inputs per level, 32 in all.
//
// Network: 32 -> 64 -> 64 -> 64 -> 1, ReLU after each hidden layer.  A CTA of 128 threads
// owns a tile of 128 samples (one per thread, one per tensor-memory lane).  Hidden layers
// are tcgen05 BF16 x BF16 -> FP32 multiplies: the tile's inputs and activations are BF16
// operand tiles in shared memory, the weights come in by one bulk copy, and the FP32
// products land in tensor memory, from where each thread reads its own sample's row, adds
// the bias and applies the ReLU.  The output layer is an FP32 dot product per thread.
//
// Training (mean squared error against clamp(d, -Clamp, Clamp)) runs the backward pass on
// the tensor cores too: dH = dZ * W reads the weight tile MN-major, and the weight
// gradients dW = dZ^T * H read the sample-major activation tiles MN-major (K = samples),
// so no transposed copies are made.  Layers 3 and 2 share one multiply: A = [dZ3 | dZ2]
// (128 rows) against B = [H2 | H1 | 1] gives dW3, dW2 and both bias gradients in its two
// diagonal blocks; layer 1 multiplies [dZ1 | .] against [X | 1].  The weight gradients
// accumulate in tensor memory over all of a CTA's tiles.
#include <cstdint>
#include <cuda_bf16.h>

#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_tc.cuh"
#include "tg_trace.cuh"

namespace tg
{
	namespace
	{
		constexpr int kRows = 128;                  // samples per tile = threads per CTA

		// ---- encoding ------------------------------------------------------------------

		__device__ __forceinline__ uint32_t CornerIndex(const FieldGrid& G, int level, uint32_t x, uint32_t y, uint32_t z)
		{
			if ((G.DenseLevels >> level) & 1u)
			{
				const uint32_t s = static_cast<uint32_t>(G.Res[level]) + 1u;
				return x + s * (y + s * z);
			}
			return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (G.TableSize - 1u);
		}

		__device__ __forceinline__ void UnitCoords(const FieldGrid& G, float x, float y, float z, float (&u)[3])
		{
			u[0] = fminf(fmaxf((x - G.Lo[0]) * G.Scale[0], 0.0f), 1.0f);
			u[1] = fminf(fmaxf((y - G.Lo[1]) * G.Scale[1], 0.0f), 1.0f);
			u[2] = fminf(fmaxf((z - G.Lo[2]) * G.Scale[2], 0.0f), 1.0f);
		}

		__device__ __forceinline__ void LevelCell(const FieldGrid& G, int l, const float (&u)[3], uint32_t (&i0)[3], float (&f)[3])
		{
			const int R = G.Res[l];
#pragma unroll
			for (int a = 0; a < 3; ++a)
			{
				const float x = u[a] * static_cast<float>(R);
				int c = static_cast<int>(floorf(x));
				c = min(max(c, 0), R - 1);
				i0[a] = static_cast<uint32_t>(c);
				f[a] = x - static_cast<float>(c);
			}
		}

		__device__ __forceinline__ float CornerWeight(int c, const float (&f)[3])
		{
			const float wx = (c & 1) ? f[0] : 1.0f - f[0];
			const float wy = (c & 2) ? f[1] : 1.0f - f[1];
			const float wz = (c & 4) ? f[2] : 1.0f - f[2];
			return (wx * wy) * wz;
		}

		// Features of levels l0 .. l0 + 3 (8 values) at unit coordinates u.
		__device__ __forceinline__ void Encode4(const FieldGrid& G, const float2* __restrict__ table, const float (&u)[3], int l0,
			float (&feat)[8])
		{
#pragma unroll
			for (int q = 0; q < 4; ++q)
			{
				const int l = l0 + q;
				uint32_t i0[3];
				float f[3];
				LevelCell(G, l, u, i0, f);
				const float2* T = table + static_cast<size_t>(l) * G.TableSize;
				float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
				for (int c = 0; c < 8; ++c)
				{
					const float w = CornerWeight(c, f);
					const float2 t = __ldg(T + CornerIndex(G, l, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + (c >> 2)));
					a0 = __fmaf_rn(w, t.x, a0);
					a1 = __fmaf_rn(w, t.y, a1);
				}
				feat[2 * q] = a0;
				feat[2 * q + 1] = a1;
			}
		}

		// All 32 features as BF16 into the thread's row of an input tile (C columns).
		__device__ __forceinline__ void EncodeRow(const FieldGrid& G, const float2* __restrict__ table, const float (&u)[3], void* tile,
			uint32_t C)
		{
#pragma unroll 1
			for (int l0 = 0; l0 < kFieldLevels; l0 += 4)
			{
				float o[8];
				Encode4(G, table, u, l0, o);
				tc::StoreRow8(tile, threadIdx.x, 2 * l0, C, o);
			}
		}

		// Adds w_corner * dfeat to the table gradient at every corner of levels l0 .. l0 + 7
		// (dfeat: those levels' 16 feature gradients).
		__device__ __forceinline__ void ScatterTableGrad8(const FieldGrid& G, float2* __restrict__ grad, const float (&u)[3], int l0,
			const float (&dfeat)[16])
		{
#pragma unroll
			for (int q = 0; q < 8; ++q)
			{
				const int l = l0 + q;
				uint32_t i0[3];
				float f[3];
				LevelCell(G, l, u, i0, f);
				float2* T = grad + static_cast<size_t>(l) * G.TableSize;
				const float g0 = dfeat[2 * q], g1 = dfeat[2 * q + 1];
#pragma unroll
				for (int c = 0; c < 8; ++c)
				{
					const float w = CornerWeight(c, f);
					atomicAdd(T + CornerIndex(G, l, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + (c >> 2)), make_float2(w * g0, w * g1));
				}
			}
		}

		// ---- tensor-core stages --------------------------------------------------------

		struct Pipe
		{
			uint64_t* Bar;        // MMA completion barrier
			uint32_t Tmem;        // allocation base
			uint32_t Phase;
		};

		// Between a stage's shared-memory writes (and tensor-memory reads) and the next
		// multiply: makes the writes visible to the tensor core, orders the reads before it,
		// and tells every thread whether any thread's last wait failed.
		__device__ __forceinline__ bool StageSync(bool failed)
		{
			tc::FenceProxyAsync();
			tc::FenceBeforeSync();
			const int any = __syncthreads_or(failed ? 1 : 0);
			tc::FenceAfterSync();
			return any != 0;
		}

		// Thread 0 (which issued the multiplies) commits; every thread waits.
		__device__ __forceinline__ bool Complete(Pipe& p)
		{
			if (threadIdx.x == 0) tc::Commit(p.Bar);
			const bool ok = tc::BarWait(p.Bar, p.Phase);
			p.Phase ^= 1u;
			tc::FenceAfterSync();
			return ok;
		}

		// Warp-uniform tensor-memory address of this warp's lanes at `column`.
		__device__ __forceinline__ uint32_t WarpTmem(const Pipe& p, uint32_t column)
		{
			return tc::TmemAddr(p.Tmem, threadIdx.x & ~31u, column);
		}

		// Hidden-layer epilogue: z = acc + bias; relu(z) as BF16 into the thread's row of
		// `tile` at columns [c0, c0 + 64).  Returns the mask of z > 0.
		__device__ __forceinline__ uint64_t HiddenEpilogue(uint32_t taddr, const float* bias, void* tile, uint32_t C, uint32_t c0)
		{
			uint64_t mask = 0;
#pragma unroll
			for (int q = 0; q < 4; ++q)
			{
				float v[16];
				tc::Load16(taddr + q * 16, v);
#pragma unroll
				for (int h = 0; h < 2; ++h)
				{
					float o[8];
#pragma unroll
					for (int i = 0; i < 8; ++i)
					{
						const int j = q * 16 + h * 8 + i;
						const float z = v[h * 8 + i] + bias[j];
						o[i] = fmaxf(z, 0.0f);
						mask |= static_cast<uint64_t>(z > 0.0f) << j;
					}
					tc::StoreRow8(tile, threadIdx.x, c0 + q * 16 + h * 8, C, o);
				}
			}
			return mask;
		}

		// Backward epilogue: dz = acc * (mask bit), BF16 into the thread's row.
		__device__ __forceinline__ void MaskEpilogue(uint32_t taddr, uint64_t mask, void* tile, uint32_t C, uint32_t c0)
		{
#pragma unroll
			for (int q = 0; q < 4; ++q)
			{
				float v[16];
				tc::Load16(taddr + q * 16, v);
#pragma unroll
				for (int h = 0; h < 2; ++h)
				{
					float o[8];
#pragma unroll
					for (int i = 0; i < 8; ++i)
					{
						const int j = q * 16 + h * 8 + i;
						o[i] = ((mask >> j) & 1u) ? v[h * 8 + i] : 0.0f;
					}
					tc::StoreRow8(tile, threadIdx.x, c0 + q * 16 + h * 8, C, o);
				}
			}
		}

		// Test hook of the network-image wait (SetSetupWaitTest): nonzero, every thread first
		// waits this long on an mbarrier that nothing arrives at (bars[2]), so Setup fails as
		// if the image copy had not completed.
		__device__ unsigned long long g_setup_wait_test_ns = 0;

		// Shared setup: tensor memory (warp 0), barriers (thread 0), the network image by one
		// bulk copy.  Returns false if the copy's wait ran out; the copy has then landed (a
		// second bounded wait) before the caller tears the CTA down.
		__device__ __forceinline__ bool Setup(uint32_t* tmem_slot, uint64_t* bars, void* image_dst, const uint8_t* image,
			uint32_t columns, Pipe& p)
		{
			if (threadIdx.x < 32) tc::Alloc(tmem_slot, columns);
			if (threadIdx.x == 0)
			{
				tc::BarInit(&bars[0], 1);
				tc::BarInit(&bars[1], 1);
				tc::BarInit(&bars[2], 1);
			}
			tc::FenceBeforeSync();
			__syncthreads();
			tc::FenceAfterSync();
			p.Tmem = *tmem_slot;
			p.Bar = &bars[1];
			p.Phase = 0;
			if (threadIdx.x == 0) tc::BulkLoad(image_dst, image, kImageBytes, &bars[0]);
			const uint64_t testLimit = g_setup_wait_test_ns;
			const bool ok = testLimit ? tc::BarWaitFor(&bars[2], 0, testLimit) : tc::BarWait(&bars[0], 0);
			if (ok) return true;
			tc::BarWait(&bars[0], 0);
			return false;
		}

		__device__ __forceinline__ void Teardown(const Pipe& p, uint32_t columns, bool failed, int* status)
		{
			if (failed && threadIdx.x == 0 && status) atomicExch(status, 1);
			tc::FenceBeforeSync();
			__syncthreads();
			if (threadIdx.x < 32)
			{
				tc::FenceAfterSync();
				tc::Dealloc(p.Tmem, columns);
			}
		}

		// ---- inference -----------------------------------------------------------------

		struct alignas(16) InferSmem
		{
			uint8_t X[kRows * 32 * 2];          // inputs, 128 x 32
			uint8_t H[kRows * 64 * 2];          // activations, 128 x 64 (H1, then H2)
			uint8_t Image[kImageBytes];
			uint64_t Bars[3];
			uint32_t TmemSlot;
		};
		constexpr uint32_t kInferColumns = 64;

		// Network output for this thread's point (all 128 threads call together).  Returns
		// false when a wait ran out (on every thread alike).
		__device__ __forceinline__ bool ForwardTile(const FieldGrid& G, const float2* __restrict__ table, InferSmem& S, Pipe& p,
			const float (&u)[3], float& out)
		{
			EncodeRow(G, table, u, S.X, 32);
			const float* tail = reinterpret_cast<const float*>(S.Image + kImageTail);
			const uint32_t id = tc::InstrBf16(128, 64, false, false);
			const uint32_t acc = WarpTmem(p, 0);

			if (StageSync(false)) return false;
			if (threadIdx.x == 0)
				for (int k = 0; k < 2; ++k) tc::Mma(p.Tmem, tc::KMajor(S.X, 32, k * 16), tc::KMajor(S.Image + kImageW1, 32, k * 16), id, k);
			bool failed = !Complete(p);
			HiddenEpilogue(acc, tail, S.H, 64, 0);

			if (StageSync(failed)) return false;
			if (threadIdx.x == 0)
				for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.H, 64, k * 16), tc::KMajor(S.Image + kImageW2, 64, k * 16), id, k);
			failed = !Complete(p);
			HiddenEpilogue(acc, tail + 64, S.H, 64, 0);

			if (StageSync(failed)) return false;
			if (threadIdx.x == 0)
				for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.H, 64, k * 16), tc::KMajor(S.Image + kImageW3, 64, k * 16), id, k);
			failed = !Complete(p);
			float s = 0.0f;
#pragma unroll
			for (int q = 0; q < 4; ++q)
			{
				float v[16];
				tc::Load16(acc + q * 16, v);
#pragma unroll
				for (int i = 0; i < 16; ++i)
				{
					const int j = q * 16 + i;
					s = __fmaf_rn(fmaxf(v[i] + tail[128 + j], 0.0f), tail[192 + j], s);
				}
			}
			out = s + tail[256];
			return !failed;
		}

		__global__ void __launch_bounds__(kRows) FieldEvalKernel(FieldGrid G, const float2* __restrict__ table,
			const uint8_t* __restrict__ image, const float* __restrict__ points, int64_t n, int stride, float* __restrict__ out, int* status)
		{
			extern __shared__ __align__(128) uint8_t smem[];
			InferSmem& S = *reinterpret_cast<InferSmem*>(smem);
			const int64_t tiles = (n + kRows - 1) / kRows;
			Pipe p;
			bool failed = !Setup(&S.TmemSlot, S.Bars, S.Image, image, kInferColumns, p);
			for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
			{
				if (StageSync(failed)) { failed = true; break; }
				const int64_t i = tile * kRows + threadIdx.x;
				const int64_t j = i < n ? i : n - 1;
				float u[3];
				UnitCoords(G, points[j * stride], points[j * stride + 1], points[j * stride + 2], u);
				float s;
				if (!ForwardTile(G, table, S, p, u, s)) { failed = true; break; }
				if (i < n) out[i] = s;
			}
			Teardown(p, kInferColumns, failed, status);
		}

		// ---- training ------------------------------------------------------------------

		constexpr uint32_t kHHCols = 144;    // [H2 | H1 | 1 | 0 ...]
		constexpr uint32_t kXCols = 48;      // [X | 1 | 0 ...]
		constexpr uint32_t kDZCols = 128;    // [dZ3 or dZ1 | dZ2]
		constexpr uint32_t kTrainColumns = 256;
		constexpr uint32_t kAccCat = 64;     // tensor-memory column of the stacked dW3/dW2 sums (144 wide)
		constexpr uint32_t kAccW1 = 208;     // column of the dW1 sums (48 wide)

		// Operand tiles first, the network image after them, then a guard: every operand the
		// tensor core reads lies inside this block however its descriptor strides are taken.
		struct alignas(16) TrainSmem
		{
			uint8_t DZ[kRows * kDZCols * 2];
			uint8_t HH[kRows * kHHCols * 2];
			uint8_t X[kRows * kXCols * 2];
			uint8_t Image[kImageBytes];
			float Out[68];                      // sums of dW4 (64) and db4, then the squared error
			uint64_t Bars[3];
			uint32_t TmemSlot;
			uint8_t Guard[8192];
		};
		static_assert(sizeof(TrainSmem) <= 113 * 1024, "two training CTAs must fit an SM");

		// Sum over the warp of v[lane >> 1]: a reduce-scatter that halves the values at each
		// of four exchange steps and finishes with a pairwise sum.
		__device__ __forceinline__ float WarpReduceScatter16(const float (&v)[16], int lane)
		{
			float a[8], b[4], c[2];
#pragma unroll
			for (int i = 0; i < 8; ++i)
			{
				const bool hi = lane & 16;
				const float send = hi ? v[i] : v[i + 8], keep = hi ? v[i + 8] : v[i];
				a[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 16);
			}
#pragma unroll
			for (int i = 0; i < 4; ++i)
			{
				const bool hi = lane & 8;
				const float send = hi ? a[i] : a[i + 4], keep = hi ? a[i + 4] : a[i];
				b[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 8);
			}
#pragma unroll
			for (int i = 0; i < 2; ++i)
			{
				const bool hi = lane & 4;
				const float send = hi ? b[i] : b[i + 2], keep = hi ? b[i + 2] : b[i];
				c[i] = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 4);
			}
			const bool hi = lane & 2;
			const float send = hi ? c[0] : c[1], keep = hi ? c[1] : c[0];
			float d = keep + __shfl_xor_sync(0xFFFFFFFFu, send, 2);
			d += __shfl_xor_sync(0xFFFFFFFFu, d, 1);
			return d;
		}

		__device__ __forceinline__ float WarpSum(float x)
		{
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
			return x;
		}

		__global__ void __launch_bounds__(kRows) FieldTrainKernel(FieldGrid G, const float2* __restrict__ table,
			const uint8_t* __restrict__ image, const float4* __restrict__ samples, int64_t n, float inv_n,
			float2* __restrict__ table_grad, float* __restrict__ mlp_grad, float* __restrict__ loss, int* status)
		{
			extern __shared__ __align__(128) uint8_t smem[];
			TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem);
			const int t = threadIdx.x, lane = t & 31;
			if (t < 68) S.Out[t] = 0.0f;
			{
				// Constant columns: X col 32 and HH col 128 are ones, the padding zeros.
				const float one[8] = { 1, 0, 0, 0, 0, 0, 0, 0 }, zero[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
				tc::StoreRow8(S.X, t, 32, kXCols, one);
				tc::StoreRow8(S.X, t, 40, kXCols, zero);
				tc::StoreRow8(S.HH, t, 128, kHHCols, one);
				tc::StoreRow8(S.HH, t, 136, kHHCols, zero);
			}
			Pipe p;
			bool failed = !Setup(&S.TmemSlot, S.Bars, S.Image, image, kTrainColumns, p);
			const float* tail = reinterpret_cast<const float*>(S.Image + kImageTail);
			const uint32_t scratch = WarpTmem(p, 0);
			const uint32_t idFwd = tc::InstrBf16(128, 64, false, false);
			const uint32_t idDH = tc::InstrBf16(128, 64, false, true);
			const uint32_t idDX = tc::InstrBf16(128, 32, false, true);
			const uint32_t idCat = tc::InstrBf16(128, kHHCols, true, true);
			const uint32_t idW1 = tc::InstrBf16(128, kXCols, true, true);
			const int64_t tiles = (n + kRows - 1) / kRows;
			uint32_t accumulated = 0;
			for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
			{
				const int64_t i = tile * kRows + t;
				const bool valid = i < n;
				const float4 smp = samples[valid ? i : n - 1];
				float u[3];
				UnitCoords(G, smp.x, smp.y, smp.z, u);
				EncodeRow(G, table, u, S.X, kXCols);
				// Forward.
				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
					for (int k = 0; k < 2; ++k) tc::Mma(p.Tmem, tc::KMajor(S.X, kXCols, k * 16), tc::KMajor(S.Image + kImageW1, 32, k * 16), idFwd, k);
				failed = !Complete(p);
				const uint64_t m1 = HiddenEpilogue(scratch, tail, S.HH, kHHCols, 64);

				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.HH, kHHCols, 64 + k * 16), tc::KMajor(S.Image + kImageW2, 64, k * 16), idFwd, k);
				failed = !Complete(p);
				const uint64_t m2 = HiddenEpilogue(scratch, tail + 64, S.HH, kHHCols, 0);

				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.HH, kHHCols, k * 16), tc::KMajor(S.Image + kImageW3, 64, k * 16), idFwd, k);
				failed = !Complete(p);
				float s = 0.0f;
#pragma unroll
				for (int q = 0; q < 4; ++q)
				{
					float v[16];
					tc::Load16(scratch + q * 16, v);
#pragma unroll
					for (int k = 0; k < 16; ++k) s = __fmaf_rn(fmaxf(v[k] + tail[128 + q * 16 + k], 0.0f), tail[192 + q * 16 + k], s);
				}
				s = s + tail[256];
				const float target = fminf(fmaxf(smp.w, -G.Clamp), G.Clamp);
				const float diff = s - target;
				const float g = valid ? 2.0f * diff * inv_n : 0.0f;
				{
					const float sq = WarpSum(valid ? diff * diff : 0.0f);
					const float gs = WarpSum(g);
					if (lane == 0)
					{
						atomicAdd(&S.Out[65], sq);
						atomicAdd(&S.Out[64], gs);
					}
				}
				// Output layer: dW4 += g h3, dZ3 = g W4 (z3 > 0).
#pragma unroll
				for (int q = 0; q < 4; ++q)
				{
					float v[16], gh[16];
					tc::Load16(scratch + q * 16, v);
#pragma unroll
					for (int h = 0; h < 2; ++h)
					{
						float o[8];
#pragma unroll
						for (int k = 0; k < 8; ++k)
						{
							const int j = q * 16 + h * 8 + k;
							const float z = v[h * 8 + k] + tail[128 + j];
							gh[h * 8 + k] = g * fmaxf(z, 0.0f);
							o[k] = z > 0.0f ? g * tail[192 + j] : 0.0f;
						}
						tc::StoreRow8(S.DZ, t, q * 16 + h * 8, kDZCols, o);
					}
					const float r = WarpReduceScatter16(gh, lane);
					if ((lane & 1) == 0) atomicAdd(&S.Out[q * 16 + (lane >> 1)], r);
				}

				// dH2 = dZ3 W3.
				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.DZ, kDZCols, k * 16), tc::MNMajor(S.Image + kImageW3, 64, k * 16), idDH, k);
				failed = !Complete(p);
				MaskEpilogue(scratch, m2, S.DZ, kDZCols, 64);            // dZ2

				// dH1 = dZ2 W2; [dW3 db3 ; dW2 db2] += [dZ3 | dZ2]^T [H2 | H1 | 1].
				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
				{
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.DZ, kDZCols, 64 + k * 16), tc::MNMajor(S.Image + kImageW2, 64, k * 16), idDH, k);
					for (int k = 0; k < 8; ++k)
						tc::Mma(p.Tmem + kAccCat, tc::MNMajor(S.DZ, kDZCols, k * 16), tc::MNMajor(S.HH, kHHCols, k * 16), idCat, (accumulated | k) ? 1u : 0u);
				}
				failed = !Complete(p);
				MaskEpilogue(scratch, m1, S.DZ, kDZCols, 0);             // dZ1

				// dX = dZ1 W1; [dW1 db1] += dZ1^T [X | 1].
				if (StageSync(failed)) { failed = true; break; }
				if (t == 0)
				{
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.DZ, kDZCols, k * 16), tc::MNMajor(S.Image + kImageW1, 32, k * 16), idDX, k);
					for (int k = 0; k < 8; ++k)
						tc::Mma(p.Tmem + kAccW1, tc::MNMajor(S.DZ, kDZCols, k * 16), tc::MNMajor(S.X, kXCols, k * 16), idW1, (accumulated | k) ? 1u : 0u);
				}
				failed = !Complete(p);
				accumulated = 1;
#pragma unroll 1
				for (int h = 0; h < 2; ++h)
				{
					float v[16];
					tc::Load16(scratch + 16 * h, v);
					if (valid && !failed) ScatterTableGrad8(G, table_grad, u, 8 * h, v);
				}
			}
			// Weight-gradient sums: lane r of the stacked block holds row r (r < 64: layer 3,
			// r >= 64: layer 2 at column offset 64); rows < 64 of the dW1 block are layer 1.
			if (!StageSync(failed) && accumulated)
			{
				const uint32_t cat = WarpTmem(p, kAccCat);
				const int row = t & 63;
				float* dW = mlp_grad + (t < 64 ? kFieldW3 : kFieldW2) + row * 64;
				const uint32_t c0 = t < 64 ? 0 : 64;
#pragma unroll
				for (int q = 0; q < 8; ++q)
				{
					float v[16];
					tc::Load16(cat + q * 16, v);
					// Columns q*16 .. q*16+15 of the block; this row's own diagonal block is
					// columns [c0, c0 + 64).
					const int col0 = q * 16;
					if (col0 >= (int)c0 && col0 < (int)c0 + 64)
					{
#pragma unroll
						for (int k = 0; k < 16; ++k) atomicAdd(dW + (col0 - (int)c0) + k, v[k]);
					}
				}
				{
					float v[16];
					tc::Load16(cat + 128, v);
					atomicAdd(mlp_grad + (t < 64 ? kFieldB3 : kFieldB2) + row, v[0]);
				}
				const uint32_t w1 = WarpTmem(p, kAccW1);
				float v0[16], v1[16], v2[16];
				tc::Load16(w1, v0);
				tc::Load16(w1 + 16, v1);
				tc::Load16(w1 + 32, v2);
				if (t < 64)
				{
#pragma unroll
					for (int k = 0; k < 16; ++k)
					{
						atomicAdd(mlp_grad + kFieldW1 + t * 32 + k, v0[k]);
						atomicAdd(mlp_grad + kFieldW1 + t * 32 + 16 + k, v1[k]);
					}
					atomicAdd(mlp_grad + kFieldB1 + t, v2[0]);
				}
				if (t < 64) atomicAdd(mlp_grad + kFieldW4 + t, S.Out[t]);
				if (t == 64) atomicAdd(mlp_grad + kFieldB4, S.Out[64]);
				if (t == 65) atomicAdd(loss, S.Out[65]);
			}
			Teardown(p, kTrainColumns, failed, status);
		}

		// ---- parameter updates and packing ---------------------------------------------

		__global__ void AdamKernel(float* __restrict__ params, float* __restrict__ grads, float* __restrict__ m, float* __restrict__ v,
			int64_t n, AdamStep s)
		{
			for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
			{
				const float g = grads[i];
				grads[i] = 0.0f;
				const float mi = s.Beta1 * m[i] + (1.0f - s.Beta1) * g;
				const float vi = s.Beta2 * v[i] + (1.0f - s.Beta2) * (g * g);
				m[i] = mi;
				v[i] = vi;
				params[i] -= s.Rate * (mi / s.Correction1) / (sqrtf(vi / s.Correction2) + s.Epsilon);
			}
		}

		// The same update four parameters at a time (16-byte loads and stores).
		__global__ void AdamKernel4(float4* __restrict__ params, float4* __restrict__ grads, float4* __restrict__ m, float4* __restrict__ v,
			int64_t n4, AdamStep s)
		{
			for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x)
			{
				const float4 g = grads[i];
				grads[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
				float4 mi = m[i], vi = v[i], p = params[i];
				float* pg = (float*)&g;
				float* pm = (float*)&mi;
				float* pv = (float*)&vi;
				float* pp = (float*)&p;
#pragma unroll
				for (int k = 0; k < 4; ++k)
				{
					pm[k] = s.Beta1 * pm[k] + (1.0f - s.Beta1) * pg[k];
					pv[k] = s.Beta2 * pv[k] + (1.0f - s.Beta2) * (pg[k] * pg[k]);
					pp[k] -= s.Rate * (pm[k] / s.Correction1) / (sqrtf(pv[k] / s.Correction2) + s.Epsilon);
				}
				m[i] = mi;
				v[i] = vi;
				params[i] = p;
			}
		}

		__global__ void FieldPackKernel(const float* __restrict__ mlp, uint8_t* __restrict__ image)
		{
			for (int e = threadIdx.x; e < 64 * 32; e += blockDim.x)
			{
				const int o = e / 32, i = e % 32;
				*reinterpret_cast<__nv_bfloat16*>(image + kImageW1 + tc::TileOffset(o, i, 32)) = __float2bfloat16_rn(mlp[kFieldW1 + e]);
			}
			for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x)
			{
				const int o = e / 64, i = e % 64;
				*reinterpret_cast<__nv_bfloat16*>(image + kImageW2 + tc::TileOffset(o, i, 64)) = __float2bfloat16_rn(mlp[kFieldW2 + e]);
				*reinterpret_cast<__nv_bfloat16*>(image + kImageW3 + tc::TileOffset(o, i, 64)) = __float2bfloat16_rn(mlp[kFieldW3 + e]);
			}
			float* tail = reinterpret_cast<float*>(image + kImageTail);
			for (int j = threadIdx.x; j < 64; j += blockDim.x)
			{
				tail[j] = mlp[kFieldB1 + j];
				tail[64 + j] = mlp[kFieldB2 + j];
				tail[128 + j] = mlp[kFieldB3 + j];
				tail[192 + j] = __bfloat162float(__float2bfloat16_rn(mlp[kFieldW4 + j]));
			}
			if (threadIdx.x == 0)
			{
				tail[256] = mlp[kFieldB4];
				tail[257] = tail[258] = tail[259] = 0.0f;
			}
		}

		// ---- training data ---------------------------------------------------------------

		// splitmix64 finaliser (Steele, Lea and Flood 2014) over a Weyl sequence.
		__device__ __forceinline__ uint64_t Mix64(uint64_t z)
		{
			z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
			z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
			return z ^ (z >> 31);
		}

		__device__ __forceinline__ float Uniform01(uint64_t seed, uint64_t counter)
		{
			return static_cast<float>(Mix64(seed + (counter + 1) * 0x9E3779B97F4A7C15ull) >> 40) * (1.0f / 16777216.0f);
		}

		__global__ void UniformKernel(uint64_t seed, float3 lo, float3 ext, float4* __restrict__ out, int64_t n, int64_t stride,
			int64_t offset)
		{
			const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (i >= n) return;
			const uint64_t c = static_cast<uint64_t>(i) * 3u;
			out[i * stride + offset] = make_float4(lo.x + ext.x * Uniform01(seed, c), lo.y + ext.y * Uniform01(seed, c + 1),
				lo.z + ext.z * Uniform01(seed, c + 2), 0.0f);
		}

		__global__ void EvalFullKernel(DeviceProgram prog, float4* __restrict__ samples, int64_t n)
		{
			const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (i >= n) return;
			float4 s = samples[i];
			s.w = RunSurface(prog.Code, prog.FullSurfaceCode, Vec3(s.x, s.y, s.z), false, nullptr);
			samples[i] = s;
		}

		__global__ void BandFlagsKernel(const float4* __restrict__ samples, int64_t n, float band, uint32_t* __restrict__ words)
		{
			const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			const bool f = i < n && fabsf(samples[i < n ? i : 0].w) < band;
			const unsigned b = __ballot_sync(0xFFFFFFFFu, f);
			if ((threadIdx.x & 31) == 0 && i < n) words[i >> 5] = b;
		}

		__global__ void BandCompactKernel(const float4* __restrict__ samples, int64_t n, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, float4* __restrict__ out, int64_t first, int64_t limit, int64_t stride, int64_t offset)
		{
			const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (i >= n) return;
			const uint32_t w = words[i >> 5];
			if (!((w >> (i & 31)) & 1u)) return;
			const int64_t r = first + base[i >> 5] + __popc(w & ((1u << (i & 31)) - 1u));
			if (r < limit) out[r * stride + offset] = samples[i];
		}

		// ---- brick culling with the network ----------------------------------------------

		struct Bricks
		{
			int B, NBX, NBY, NBZ;
		};

		// One network evaluation per brick centre, 128 bricks per tile.
		__global__ void __launch_bounds__(kRows) FieldClassifyKernel(DeviceProgram prog, GridSpec g, Bricks bg, FieldGrid G,
			const float2* __restrict__ table, const uint8_t* __restrict__ image, float margin, uint32_t* __restrict__ brick_bits,
			int* status)
		{
			extern __shared__ __align__(128) uint8_t smem[];
			InferSmem& S = *reinterpret_cast<InferSmem*>(smem);
			const int64_t nb = (int64_t)bg.NBX * bg.NBY * bg.NBZ;
			const int64_t tiles = (nb + kRows - 1) / kRows;
			Pipe p;
			bool failed = !Setup(&S.TmemSlot, S.Bars, S.Image, image, kInferColumns, p);
			const float rootClip = fabsf(__ldg(&prog.Nodes[0].ClipRadius));
			const float half = rootClip * 0.57736f;
			const float rx = __ldg(&prog.Nodes[0].Pivot[0]), ry = __ldg(&prog.Nodes[0].Pivot[1]), rz = __ldg(&prog.Nodes[0].Pivot[2]);
			for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
			{
				if (StageSync(failed)) { failed = true; break; }
				const int64_t b = tile * kRows + threadIdx.x;
				const int64_t bc = b < nb ? b : nb - 1;
				const int bx = (int)(bc % bg.NBX), by = (int)((bc / bg.NBX) % bg.NBY), bz = (int)(bc / ((int64_t)bg.NBX * bg.NBY));
				const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
				const int i1 = min(i0 + bg.B, g.NX - 1), j1 = min(j0 + bg.B, g.NY - 1), k1 = min(k0 + bg.B, g.NZ - 1);
				const float x0 = LatticeCoord(g.X0, i0, g.DX), x1 = LatticeCoord(g.X0, i1, g.DX);
				const float y0 = LatticeCoord(g.Y0, j0, g.DY), y1 = LatticeCoord(g.Y0, j1, g.DY);
				const float z0 = LatticeCoord(g.Z0, k0, g.DZ), z1 = LatticeCoord(g.Z0, k1, g.DZ);
				const float cx = 0.5f * (x0 + x1), cy = 0.5f * (y0 + y1), cz = 0.5f * (z0 + z1);
				const float ex = 0.5f * (x1 - x0), ey = 0.5f * (y1 - y0), ez = 0.5f * (z1 - z0);
				const float r = sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f + 1e-6f;
				const float slack = 1e-4f * (1.0f + fabsf(cx) + fabsf(cy) + fabsf(cz) + rootClip);
				float u[3];
				UnitCoords(G, cx, cy, cz, u);
				float s;
				if (!ForwardTile(G, table, S, p, u, s)) { failed = true; break; }
				const float ox = fmaxf(fabsf(cx - rx) - half, 0.0f), oy = fmaxf(fabsf(cy - ry) - half, 0.0f), oz = fmaxf(fabsf(cz - rz) - half, 0.0f);
				const bool outsideRoot = sqrtf(ox * ox + oy * oy + oz * oz) > r + slack;
				const bool inDomain = (cx - G.Lo[0]) * G.Scale[0] >= 0.0f && (cx - G.Lo[0]) * G.Scale[0] <= 1.0f &&
					(cy - G.Lo[1]) * G.Scale[1] >= 0.0f && (cy - G.Lo[1]) * G.Scale[1] <= 1.0f &&
					(cz - G.Lo[2]) * G.Scale[2] >= 0.0f && (cz - G.Lo[2]) * G.Scale[2] <= 1.0f;
				const bool ruledOut = prog.Lipschitz && inDomain && fabsf(s) > r + margin + slack;
				const bool active = b < nb && !outsideRoot && !ruledOut;
				const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
				if ((threadIdx.x & 31) == 0 && b < nb) brick_bits[b >> 5] = ballot;
			}
			Teardown(p, kInferColumns, failed, status);
		}

		// ---- sphere tracing with network steps ------------------------------------------
		//
		// Approach: a CTA marches 128 rays (one per thread) in lockstep; every iteration the
		// network runs once at all of them (one tensor-core tile).  A ray steps by the larger
		// of two lower bounds of the whole tree's distance: the distance to the root cube, and
		// the network's value less `margin` (safety x its largest held-out error).  When that
		// bound falls to `switch_at` the ray stops and records where (travel, iterations
		// used); a ray that leaves the root sphere has missed.  Finish (a separate, lighter
		// kernel with many more resident warps for the divergent part): the reference's exact
		// steps (SDFNode::RayMarch on the whole tree) from there, so every hit is the exact
		// program's, shaded with the whole tree's gradient and material.  The step budget is
		// shared: network iterations plus exact steps never exceed `steps`.
		__device__ __forceinline__ Vec3 PixelRay(const CameraBasis& cam, int x, int y, int width, int height, Vec3& start)
		{
			const float u = ((2.0f * ((float)x + 0.5f) / (float)width) - 1.0f) * cam.TanHalfFov * cam.Aspect;
			const float v = (1.0f - 2.0f * ((float)y + 0.5f) / (float)height) * cam.TanHalfFov;
			const Vec3 fwd(cam.Forward[0], cam.Forward[1], cam.Forward[2]);
			const Vec3 right(cam.Right[0], cam.Right[1], cam.Right[2]);
			const Vec3 up(cam.Up[0], cam.Up[1], cam.Up[2]);
			start = Vec3(cam.Position[0], cam.Position[1], cam.Position[2]);
			return Normalize((fwd + right * u) + up * v);
		}

		__global__ void __launch_bounds__(kRows) ApproachFieldKernel(DeviceProgram prog, const CameraBasis* __restrict__ cams, int count,
			int width, int height, int steps, FieldGrid G, const float2* __restrict__ table, const uint8_t* __restrict__ image,
			float margin, float switch_at, float* __restrict__ travel_out, uint32_t* __restrict__ state_out,
			unsigned long long* __restrict__ counters, int* status)
		{
			extern __shared__ __align__(128) uint8_t smem[];
			InferSmem& S = *reinterpret_cast<InferSmem*>(smem);
			const int64_t pixels = (int64_t)width * height;
			const int64_t total = pixels * count;
			const int64_t tiles = (total + kRows - 1) / kRows;
			Pipe p;
			bool failed = !Setup(&S.TmemSlot, S.Bars, S.Image, image, kInferColumns, p);
			unsigned long long netSteps = 0;
			for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x)
			{
				if (StageSync(failed)) { failed = true; break; }
				const int64_t t = tile * kRows + threadIdx.x;
				const bool valid = t < total;
				const int64_t tc = valid ? t : total - 1;
				const int c = (int)(tc / pixels);
				const int64_t pix = tc % pixels;
				Vec3 start;
				const Vec3 dir = PixelRay(cams[c], (int)(pix % width), (int)(pix / width), width, height, start);
				const float exitTravel = RootSphereExit(prog, start, dir);
				int mode = (valid && exitTravel >= 0.0f) ? 0 : 2;        // 0 network steps, 1 exact steps next, 2 missed
				float travel = 0.0f;
				int used = 0;
				for (int it = 0; it < steps; ++it)
				{
					if (!__syncthreads_or(mode == 0)) break;
					const Vec3 pos = dir * travel + start;
					float uu[3];
					UnitCoords(G, pos.x, pos.y, pos.z, uu);
					float s;
					if (!ForwardTile(G, table, S, p, uu, s)) { failed = true; break; }
					if (mode != 0) continue;
					++used;
					const bool inDomain = (pos.x - G.Lo[0]) * G.Scale[0] >= 0.0f && (pos.x - G.Lo[0]) * G.Scale[0] <= 1.0f &&
						(pos.y - G.Lo[1]) * G.Scale[1] >= 0.0f && (pos.y - G.Lo[1]) * G.Scale[1] <= 1.0f &&
						(pos.z - G.Lo[2]) * G.Scale[2] >= 0.0f && (pos.z - G.Lo[2]) * G.Scale[2] <= 1.0f;
					const float bound = fmaxf(RootCubeDistance(prog, pos), inDomain && prog.Lipschitz ? s - margin : 0.0f);
					if (bound > switch_at)
					{
						travel = travel + bound;
						if (travel > exitTravel) mode = 2;
					}
					else mode = 1;
				}
				if (failed) break;
				netSteps += (unsigned long long)used;
				if (valid)
				{
					travel_out[t] = travel;
					state_out[t] = (uint32_t)used | ((uint32_t)mode << 16);
				}
			}
			if (counters) atomicAdd(counters, netSteps);
			Teardown(p, kInferColumns, failed, status);
		}

		constexpr int kFinishThreads = 128;

		__global__ void __launch_bounds__(kFinishThreads) FinishFieldKernel(DeviceProgram prog, const CameraBasis* __restrict__ cams,
			int count, int width, int height, int steps, float epsilon, const float* __restrict__ travel_in,
			const uint32_t* __restrict__ state_in, float* __restrict__ depth, float* __restrict__ normals, uint8_t* __restrict__ colors,
			unsigned long long* __restrict__ counters)
		{
			extern __shared__ float spill[];
			const int64_t pixels = (int64_t)width * height;
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			const bool valid = t < pixels * count;
			unsigned exactSteps = 0;
			if (valid)
			{
				const int c = (int)(t / pixels);
				const int64_t pix = t % pixels;
				Vec3 start;
				const Vec3 dir = PixelRay(cams[c], (int)(pix % width), (int)(pix / width), width, height, start);
				const uint32_t state = state_in[t];
				const int used = (int)(state & 0xFFFFu), mode = (int)(state >> 16);
				float travel = travel_in[t];
				bool hit = false;
				Vec3 hitPos(0.0f, 0.0f, 0.0f);
				if (mode == 1)
				{
					const float exitTravel = RootSphereExit(prog, start, dir);
					Vec3 pos = dir * travel + start;
					for (int i = used; i < steps; ++i)
					{
						const float d = TraceSurfaceAt(prog, prog.FullSurfaceCode, pos, false, nullptr, spill + threadIdx.x, kFinishThreads);
						++exactSteps;
						if (d <= epsilon) { hit = true; hitPos = pos; break; }
						travel = travel + d;
						if (travel > exitTravel) break;
						pos = dir * travel + start;
					}
				}
				Vec3 n(0.0f, 0.0f, 0.0f);
				uchar4 col = make_uchar4(0, 0, 0, 0);
				if (hit)
				{
					int mat = -1;
					n = TraceShade(prog, prog.FullSurfaceCode, hitPos, colors != nullptr, &mat, spill + threadIdx.x, kFinishThreads);
					col = mat >= 0 ? prog.Colors[mat] : make_uchar4(255, 255, 255, 255);
				}
				depth[t] = hit ? travel : INFINITY;
				normals[t * 3] = n.x;
				normals[t * 3 + 1] = n.y;
				normals[t * 3 + 2] = n.z;
				if (colors)
				{
					colors[t * 3] = col.x;
					colors[t * 3 + 1] = col.y;
					colors[t * 3 + 2] = col.z;
				}
			}
			// One atomic per warp (blocks are whole warps; every lane gets here).
			const unsigned w = __reduce_add_sync(0xFFFFFFFFu, exactSteps);
			if (counters && (threadIdx.x & 31) == 0 && w) atomicAdd(counters + 1, (unsigned long long)w);
		}


		// ---- operand-layout check --------------------------------------------------------

		struct alignas(16) DebugSmem
		{
			uint8_t A[65536];
			uint8_t B[73728];
			uint64_t Bars[2];
			uint32_t TmemSlot;
		};

		__global__ void __launch_bounds__(kRows) DebugMmaKernel(int mode, const float* __restrict__ a, const float* __restrict__ b,
			float* __restrict__ d, int* status)
		{
			extern __shared__ __align__(128) uint8_t smem[];
			DebugSmem& S = *reinterpret_cast<DebugSmem*>(smem);
			const int t = threadIdx.x;
			const int aCols = mode == 1 ? 128 : 64;
			const int bRows = mode == 1 ? 128 : 64, bCols = mode == 1 ? 144 : 64;
			for (int c = 0; c < aCols; c += 8)
			{
				float o[8];
				for (int k = 0; k < 8; ++k) o[k] = a[t * aCols + c + k];
				tc::StoreRow8(S.A, t, c, aCols, o);
			}
			if (t < bRows)
			{
				for (int c = 0; c < bCols; c += 8)
				{
					float o[8];
					for (int k = 0; k < 8; ++k) o[k] = b[t * bCols + c + k];
					tc::StoreRow8(S.B, t, c, bCols, o);
				}
			}
			if (t < 32) tc::Alloc(&S.TmemSlot, 256);
			if (t == 0) tc::BarInit(&S.Bars[0], 1);
			tc::FenceProxyAsync();
			tc::FenceBeforeSync();
			__syncthreads();
			tc::FenceAfterSync();
			Pipe p{ &S.Bars[0], S.TmemSlot, 0 };
			const int N = mode == 1 ? 144 : 64;
			if (t == 0)
			{
				if (mode == 0)
				{
					const uint32_t id = tc::InstrBf16(128, 64, false, false);
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.A, 64, k * 16), tc::KMajor(S.B, 64, k * 16), id, k);
				}
				else if (mode == 1)
				{
					const uint32_t id = tc::InstrBf16(128, 144, true, true);
					for (int k = 0; k < 8; ++k) tc::Mma(p.Tmem, tc::MNMajor(S.A, 128, k * 16), tc::MNMajor(S.B, 144, k * 16), id, k);
				}
				else
				{
					const uint32_t id = tc::InstrBf16(128, 64, false, true);
					for (int k = 0; k < 4; ++k) tc::Mma(p.Tmem, tc::KMajor(S.A, 64, k * 16), tc::MNMajor(S.B, 64, k * 16), id, k);
				}
			}
			const bool ok = Complete(p);
			if (ok)
			{
				const uint32_t acc = WarpTmem(p, 0);
				for (int q = 0; q < N / 16; ++q)
				{
					float v[16];
					tc::Load16(acc + q * 16, v);
					for (int k = 0; k < 16; ++k) d[t * N + q * 16 + k] = v[k];
				}
			}
			Teardown(p, 256, !ok, status);
		}

		int SmCount()
		{
			static int sms = 0;
			if (sms == 0)
			{
				int dev = 0;
				cudaGetDevice(&dev);
				cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
				if (sms <= 0) sms = 1;
			}
			return sms;
		}

		template<typename Kernel>
		cudaError_t AllowSmem(Kernel k, size_t bytes)
		{
			return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
		}

		int Blocks(int64_t n, int threads)
		{
			return (int)((n + threads - 1) / threads);
		}
	}

	cudaError_t LaunchFieldPack(const float* mlp, uint8_t* image, cudaStream_t stream)
	{
		FieldPackKernel<<<1, 256, 0, stream>>>(mlp, image);
		return cudaGetLastError();
	}

	cudaError_t LaunchFieldEval(const FieldGrid& grid, const float2* table, const uint8_t* image, const float* points, int64_t n,
		int stride, float* out, int* status, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		cudaError_t e = AllowSmem(FieldEvalKernel, sizeof(InferSmem));
		if (e != cudaSuccess) return e;
		const int64_t tiles = (n + kRows - 1) / kRows;
		const int blocks = (int)(tiles < (int64_t)SmCount() * 4 ? tiles : (int64_t)SmCount() * 4);
		FieldEvalKernel<<<blocks, kRows, sizeof(InferSmem), stream>>>(grid, table, image, points, n, stride, out, status);
		return cudaGetLastError();
	}

	cudaError_t LaunchFieldTrain(const FieldGrid& grid, const float2* table, const uint8_t* image, const float4* samples, int64_t n,
		float2* table_grad, float* mlp_grad, float* loss, int* status, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		cudaError_t e = AllowSmem(FieldTrainKernel, sizeof(TrainSmem));
		if (e != cudaSuccess) return e;
		const int64_t tiles = (n + kRows - 1) / kRows;
		const int blocks = (int)(tiles < (int64_t)SmCount() * 2 ? tiles : (int64_t)SmCount() * 2);
		FieldTrainKernel<<<blocks, kRows, sizeof(TrainSmem), stream>>>(grid, table, image, samples, n, 1.0f / (float)n, table_grad,
			mlp_grad, loss, status);
		return cudaGetLastError();
	}

	cudaError_t LaunchAdam(float* params, float* grads, float* m, float* v, int64_t n, const AdamStep& step, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		const bool aligned = ((uintptr_t)params | (uintptr_t)grads | (uintptr_t)m | (uintptr_t)v) % 16 == 0;
		if (aligned && n % 4 == 0)
		{
			const int64_t n4 = n / 4;
			const int64_t want4 = (n4 + 255) / 256;
			const int blocks4 = (int)(want4 < (int64_t)SmCount() * 16 ? want4 : (int64_t)SmCount() * 16);
			AdamKernel4<<<blocks4, 256, 0, stream>>>((float4*)params, (float4*)grads, (float4*)m, (float4*)v, n4, step);
			return cudaGetLastError();
		}
		const int64_t want = (n + 255) / 256;
		const int blocks = (int)(want < (int64_t)SmCount() * 8 ? want : (int64_t)SmCount() * 8);
		AdamKernel<<<blocks, 256, 0, stream>>>(params, grads, m, v, n, step);
		return cudaGetLastError();
	}

	cudaError_t LaunchFieldUniform(uint64_t seed, const float* lo, const float* hi, float4* out, int64_t n, int64_t stride,
		int64_t offset, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		UniformKernel<<<Blocks(n, 256), 256, 0, stream>>>(seed, make_float3(lo[0], lo[1], lo[2]),
			make_float3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]), out, n, stride, offset);
		return cudaGetLastError();
	}

	cudaError_t SetSetupWaitTest(uint64_t limit_ns)
	{
		const unsigned long long v = limit_ns;
		return cudaMemcpyToSymbol(g_setup_wait_test_ns, &v, sizeof(v));
	}

	cudaError_t LaunchEvalFull(const DeviceProgram& prog, float4* samples, int64_t n, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		EvalFullKernel<<<Blocks(n, 128), 128, 0, stream>>>(prog, samples, n);
		return cudaGetLastError();
	}

	cudaError_t LaunchBandFlags(const float4* samples, int64_t n, float band, uint32_t* words, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		BandFlagsKernel<<<Blocks(n, 256), 256, 0, stream>>>(samples, n, band, words);
		return cudaGetLastError();
	}

	cudaError_t LaunchBandCompact(const float4* samples, int64_t n, const uint32_t* words, const uint32_t* word_base,
		float4* out, int64_t first, int64_t limit, int64_t stride, int64_t offset, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		BandCompactKernel<<<Blocks(n, 256), 256, 0, stream>>>(samples, n, words, word_base, out, first, limit, stride, offset);
		return cudaGetLastError();
	}

	cudaError_t LaunchFieldClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, const FieldGrid& grid,
		const float2* table, const uint8_t* image, float margin, uint32_t* brick_bits, int* status, cudaStream_t stream)
	{
		const Bricks bg{ B, (g.NX - 1 + B - 1) / B, (g.NY - 1 + B - 1) / B, (g.NZ - 1 + B - 1) / B };
		const int64_t nb = (int64_t)bg.NBX * bg.NBY * bg.NBZ;
		if (nb <= 0) return cudaSuccess;
		cudaError_t e = AllowSmem(FieldClassifyKernel, sizeof(InferSmem));
		if (e != cudaSuccess) return e;
		const int64_t tiles = (nb + kRows - 1) / kRows;
		const int blocks = (int)(tiles < (int64_t)SmCount() * 4 ? tiles : (int64_t)SmCount() * 4);
		FieldClassifyKernel<<<blocks, kRows, sizeof(InferSmem), stream>>>(prog, g, bg, grid, table, image, margin, brick_bits, status);
		return cudaGetLastError();
	}

	cudaError_t LaunchRenderField(const DeviceProgram& prog, const CameraBasis* cameras, int count, int width, int height, int steps,
		float epsilon, const FieldGrid& grid, const float2* table, const uint8_t* image, float margin, float switch_at, float* travel,
		uint32_t* state, float* depth, float* normals, uint8_t* colors, unsigned long long* counters, int* status, cudaStream_t stream)
	{
		const int64_t total = (int64_t)width * height * count;
		if (total <= 0) return cudaSuccess;
		cudaError_t e = AllowSmem(ApproachFieldKernel, sizeof(InferSmem));
		if (e != cudaSuccess) return e;
		const int64_t tiles = (total + kRows - 1) / kRows;
		const int blocks = (int)(tiles < (int64_t)SmCount() * 4 ? tiles : (int64_t)SmCount() * 4);
		ApproachFieldKernel<<<blocks, kRows, sizeof(InferSmem), stream>>>(prog, cameras, count, width, height, steps, grid, table, image,
			margin, switch_at, travel, state, counters, status);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		const int depthStack = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depthStack * 2 * kFinishThreads * sizeof(float);
		if (smem > 48 * 1024)
		{
			e = AllowSmem(FinishFieldKernel, smem);
			if (e != cudaSuccess) return e;
		}
		FinishFieldKernel<<<(unsigned)((total + kFinishThreads - 1) / kFinishThreads), kFinishThreads, smem, stream>>>(prog, cameras,
			count, width, height, steps, epsilon, travel, state, depth, normals, colors, counters);
		return cudaGetLastError();
	}

	cudaError_t LaunchDebugMma(int mode, const float* a, const float* b, float* d, int* status, cudaStream_t stream)
	{
		if (mode < 0 || mode > 2) return cudaErrorInvalidValue;
		cudaError_t e = AllowSmem(DebugMmaKernel, sizeof(DebugSmem));
		if (e != cudaSuccess) return e;
		DebugMmaKernel<<<1, kRows, sizeof(DebugSmem), stream>>>(mode, a, b, d, status);
		return cudaGetLastError();
	}
}
