// Distance evaluation over the export lattice.
//
// One CTA covers an 8 x 16 patch of lattice columns and K consecutive z levels; every
// thread evaluates its K points with one pass over the record stream of the octree cell
// they fall in (the common case: K points, one cell).  Records are read through the
// read-only cache with warp-uniform addresses, so each record quad is one broadcast
// load per warp.  Operands below the top of the postfix stack spill to shared memory in
// a thread-interleaved layout (no bank conflicts).
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_pair.cuh"

namespace tg
{
	namespace
	{
		constexpr int kTileX = 8;
		constexpr int kTileY = 16;
		constexpr int kThreads = kTileX * kTileY;

		template<int K>
		__global__ void __launch_bounds__(kThreads) EvalGridKernel(DeviceProgram prog, GridSpec g, float* __restrict__ out)
		{
			extern __shared__ float spill[];
			const int tx = threadIdx.x % kTileX;
			const int ty = threadIdx.x / kTileX;
			const int ix = blockIdx.x * kTileX + tx;
			const int iy = blockIdx.y * kTileY + ty;
			const int iz0 = blockIdx.z * K;
			const bool inPlane = ix < g.NX && iy < g.NY;
			const float x = LatticeCoord(g.X0, ix < g.NX ? ix : g.NX - 1, g.DX);
			const float y = LatticeCoord(g.Y0, iy < g.NY ? iy : g.NY - 1, g.DY);

			float px[K], py[K], pz[K], res[K];
			int cell[K];
			unsigned todo = 0;
#pragma unroll
			for (int k = 0; k < K; ++k)
			{
				const int iz = iz0 + k;
				px[k] = x;
				py[k] = y;
				pz[k] = LatticeCoord(g.Z0, iz < g.NZ ? iz : g.NZ - 1, g.DZ);
				cell[k] = DescendOctree(prog.Nodes, px[k], py[k], pz[k]);
				res[k] = 0.0f;
				if (inPlane && iz < g.NZ) todo |= 1u << k;
			}

			// Evaluate once per distinct octree cell among this thread's points.
			while (todo)
			{
				int c = -1;
#pragma unroll
				for (int k = 0; k < K; ++k)
					if (c < 0 && ((todo >> k) & 1u)) c = cell[k];
				float r[K];
				if constexpr (K % 2 == 0)
				{
					// Points in pairs through the paired FP32 instructions (tg_pair.cuh).
					const float4* code = prog.Code;
					RunDistancePaired<K>([&](int q) { return __ldg(code + q); }, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r,
						spill + 2 * threadIdx.x, kThreads);
				}
				else
				{
					RunDistance<K>(prog.Code, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r, spill + threadIdx.x, kThreads);
				}
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					if (((todo >> k) & 1u) && cell[k] == c)
					{
						res[k] = r[k];
						todo &= ~(1u << k);
					}
				}
			}

			if (inPlane)
			{
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					const int iz = iz0 + k;
					if (iz < g.NZ) out[((int64_t)iz * g.NY + iy) * g.NX + ix] = res[k];
				}
			}
		}
	}

	namespace
	{
		template<int K>
		cudaError_t LaunchEvalGridK(const DeviceProgram& prog, const GridSpec& grid, float* out, cudaStream_t stream)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			const size_t smem = (size_t)depth * K * kThreads * sizeof(float);
			if (smem > 48 * 1024)
			{
				cudaError_t e = cudaFuncSetAttribute(EvalGridKernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
				if (e != cudaSuccess) return e;
			}
			const dim3 blocks((grid.NX + kTileX - 1) / kTileX, (grid.NY + kTileY - 1) / kTileY, (grid.NZ + K - 1) / K);
			EvalGridKernel<K><<<blocks, kThreads, smem, stream>>>(prog, grid, out);
			return cudaGetLastError();
		}
	}

	cudaError_t LaunchEvalGrid(const DeviceProgram& prog, const GridSpec& grid, float* out, cudaStream_t stream, int lanes)
	{
		switch (lanes)
		{
		case 1: return LaunchEvalGridK<1>(prog, grid, out, stream);
		case 2: return LaunchEvalGridK<2>(prog, grid, out, stream);
		default: return LaunchEvalGridK<4>(prog, grid, out, stream);
		}
	}
}
