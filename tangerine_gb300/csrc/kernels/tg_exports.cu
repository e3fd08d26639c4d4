// The reference's other two lattice exports on the GPU:
//  * PointCloudExportThread (tangerine/export.cpp:384-480): voxel centres whose octree
//    distance is within the half-voxel diagonal, then gradient steps toward the surface
//    kept inside the voxel;
//  * VoxExport (tangerine/magica.cpp:27-72): voxels whose centre's full-tree distance is
//    within the half-voxel radius.
// Both keep the reference's float operation order, so the kept cells and refined points are
// the reference's bit for bit; the kept cells become an index-ordered list through the
// bitmask + scan of the brick lists.
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_surface.cuh"

namespace tg
{
	namespace
	{
		inline unsigned Blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

		// Cell i's centre: float(i / slice) * step.z + start.z (and so on), then + half.
		__device__ __forceinline__ Vec3 CloudCentre(const CloudSpec& s, int i)
		{
			const int slice = s.IX * s.IY;
			const float Z = (float)(i / slice) * s.Step[2] + s.Start[2];
			const float Y = (float)((i % slice) / s.IX) * s.Step[1] + s.Start[1];
			const float X = (float)(i % s.IX) * s.Step[0] + s.Start[0];
			return Vec3(X, Y, Z) + Vec3(s.Half[0], s.Half[1], s.Half[2]);
		}

		__device__ __forceinline__ float OctreeDistance(const DeviceProgram& prog, Vec3 p)
		{
			float spill[kMaxStack];
			const float px[1] = { p.x }, py[1] = { p.y }, pz[1] = { p.z };
			float r[1];
			const int cell = DescendOctree(prog.Nodes, p.x, p.y, p.z);
			RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, r, spill, 1);
			return r[0];
		}

		// abs(Octree->Eval(Cursor)) < Diagonal per voxel centre (export.cpp:404-423).
		__global__ void __launch_bounds__(128) CloudFlagsKernel(DeviceProgram prog, CloudSpec s, uint32_t* __restrict__ words)
		{
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool keep = false;
			if (t < s.Total)
			{
				const float d = OctreeDistance(prog, CloudCentre(s, (int)t));
				keep = fabsf(d) < s.Diagonal;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, keep);
			if ((threadIdx.x & 31) == 0 && t < s.Total) words[t >> 5] = ballot;
		}

		// SDFOctree::Gradient (the selected cell's SDFNode::Gradient, sdf_evaluator.cpp:298-333)
		// at p: the four tetrahedral evaluations share one pass over the cell's surface
		// program; the evaluation at p itself is needed only when they cancel.
		__device__ __forceinline__ Vec3 OctreeGradient(const DeviceProgram& prog, Vec3 p, float* spill)
		{
			const int cell = DescendOctree(prog.Nodes, p.x, p.y, p.z);
			const int pc = __ldg(&prog.Nodes[cell].SurfaceCode);
			float px[4], py[4], pz[4];
#pragma unroll
			for (int k = 0; k < 4; ++k)
			{
				const Vec3 q = TetraPoint(p, k);
				px[k] = q.x; py[k] = q.y; pz[k] = q.z;
			}
			float e[5];
			float r4[4];
			RunSurfaceBatch<4>(prog.Code, pc, px, py, pz, r4, -1, nullptr, spill, 1);
#pragma unroll
			for (int k = 0; k < 4; ++k) e[k] = r4[k];
			e[4] = 0.0f;
			const float h = 0.0001f;
			const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
			Vec3 g = xyy * e[0];
			g = g + yyx * e[1];
			g = g + yxy * e[2];
			g = g + xxx * e[3];
			if ((g.x * g.x + g.y * g.y) + g.z * g.z == 0.0f)
			{
				const float qx[1] = { p.x }, qy[1] = { p.y }, qz[1] = { p.z };
				float r1[1];
				RunSurfaceBatch<1>(prog.Code, pc, qx, qy, qz, r1, -1, nullptr, spill, 1);
				e[4] = r1[0];
			}
			return GradientOf(e);
		}

		// The refinement (export.cpp:434-465): `iterations` steps of Cursor += Gradient *
		// -Eval, clamped to the voxel; the point moves only if it stays within the diagonal.
		__global__ void __launch_bounds__(128) CloudRefineKernel(DeviceProgram prog, CloudSpec s, const uint32_t* __restrict__ cells,
			const uint32_t* __restrict__ count, int iterations, float* __restrict__ points)
		{
			const uint32_t n = __ldg(count);
			const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
			if (v >= n) return;
			const Vec3 vertex = CloudCentre(s, (int)__ldg(cells + v));
			const Vec3 half(s.Half[0], s.Half[1], s.Half[2]);
			Vec3 cursor = vertex;
			if (iterations > 0)
			{
				float spill[kMaxStack * 5];
				const Vec3 low = vertex - half, high = vertex + half;
				for (int r = 0; r < iterations; ++r)
				{
					const Vec3 dir = OctreeGradient(prog, cursor, spill);
					// Octree->Eval(Cursor) * -1.0 rounds back to float exactly: a negation.
					const float dist = -OctreeDistance(prog, cursor);
					cursor = cursor + dir * dist;
				}
				cursor = TernaryMin(TernaryMax(cursor, low), high);
				const Vec3 d = vertex - cursor;
				if (!(sqrtf(Dot(d, d)) <= s.Diagonal)) cursor = vertex;
			}
			points[(int64_t)v * 3 + 0] = cursor.x;
			points[(int64_t)v * 3 + 1] = cursor.y;
			points[(int64_t)v * 3 + 2] = cursor.z;
		}

		// glm::mix(x, y, a) = x * (1 - a) + y * a, per component.
		__device__ __forceinline__ float Mix(float x, float y, float a)
		{
			return x * (1.0f - a) + y * a;
		}

		// VoxExport's test (magica.cpp:52-64): the voxel centre mix(Min, Max, (x + .5) / Size)
		// on the whole tree (SDFNode::Eval), kept when |d| <= Radius.
		__global__ void __launch_bounds__(128) VoxFlagsKernel(DeviceProgram prog, VoxSpec s, uint32_t* __restrict__ words)
		{
			extern __shared__ float spill[];
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool keep = false;
			if (t < s.Total)
			{
				const int i = (int)t;
				const int slice = s.SX * s.SY;
				const int z = i / slice, y = (i % slice) / s.SX, x = i % s.SX;
				// vec3(x + .5, ...) converts the double sums to float.
				const float ax = (float)((double)x + 0.5) / (float)s.SX;
				const float ay = (float)((double)y + 0.5) / (float)s.SY;
				const float az = (float)((double)z + 0.5) / (float)s.SZ;
				const float px[1] = { Mix(s.Min[0], s.Max[0], ax) };
				const float py[1] = { Mix(s.Min[1], s.Max[1], ay) };
				const float pz[1] = { Mix(s.Min[2], s.Max[2], az) };
				float r[1];
				RunSurfaceBatch<1>(prog.Code, prog.FullSurfaceCode, px, py, pz, r, -1, nullptr, spill + threadIdx.x, 128);
				keep = fabsf(r[0]) <= s.Radius;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, keep);
			if ((threadIdx.x & 31) == 0 && t < s.Total) words[t >> 5] = ballot;
		}
	}

	cudaError_t LaunchCloudFlags(const DeviceProgram& prog, const CloudSpec& s, uint32_t* words, cudaStream_t stream)
	{
		if (s.Total <= 0) return cudaSuccess;
		CloudFlagsKernel<<<Blocks(s.Total, 128), 128, 0, stream>>>(prog, s, words);
		return cudaGetLastError();
	}

	cudaError_t LaunchCloudRefine(const DeviceProgram& prog, const CloudSpec& s, const uint32_t* cells, const uint32_t* count,
		uint32_t capacity, int iterations, float* points, cudaStream_t stream)
	{
		if (capacity == 0) return cudaSuccess;
		CloudRefineKernel<<<Blocks(capacity, 128), 128, 0, stream>>>(prog, s, cells, count, iterations, points);
		return cudaGetLastError();
	}

	cudaError_t LaunchVoxFlags(const DeviceProgram& prog, const VoxSpec& s, uint32_t* words, cudaStream_t stream)
	{
		if (s.Total <= 0) return cudaSuccess;
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depth * 2 * 128 * sizeof(float);
		if (smem > 48 * 1024)
		{
			cudaError_t e = cudaFuncSetAttribute(VoxFlagsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		VoxFlagsKernel<<<Blocks(s.Total, 128), 128, smem, stream>>>(prog, s, words);
		return cudaGetLastError();
	}
}
