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

		// `spill`: this thread's column of the operand stack in shared memory (stride
		// `stride`), as the interpreters lay it out.
		__device__ __forceinline__ float OctreeDistance(const DeviceProgram& prog, Vec3 p, float* spill, int stride)
		{
			const float px[1] = { p.x }, py[1] = { p.y }, pz[1] = { p.z };
			float r[1];
			const int cell = DescendOctree(prog.Nodes, p.x, p.y, p.z);
			RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, r, spill, stride);
			return r[0];
		}

		// Voxel bricks: 8^3 voxels whose tests are decided together when a bound proves that
		// none of them can pass.  The distance functions are 1-Lipschitz (or the test is not
		// made), so |f(c)| > r + threshold + margin at the centre c of the ball (radius r)
		// through the brick's voxel centres means |f| > threshold at every one of them; the
		// margin covers the rounding of f at c and at the voxel (as in the export's bricks).
		constexpr int kVoxelBrick = 8;

		struct VoxelBricks
		{
			int NX, NY, NZ;     // bricks per axis
		};

		__device__ __forceinline__ void BrickRange(int b, const VoxelBricks& vb, int sx, int sy, int sz, int (&lo)[3], int (&hi)[3])
		{
			const int bx = b % vb.NX, by = (b / vb.NX) % vb.NY, bz = b / (vb.NX * vb.NY);
			lo[0] = bx * kVoxelBrick; hi[0] = min(lo[0] + kVoxelBrick - 1, sx - 1);
			lo[1] = by * kVoxelBrick; hi[1] = min(lo[1] + kVoxelBrick - 1, sy - 1);
			lo[2] = bz * kVoxelBrick; hi[2] = min(lo[2] + kVoxelBrick - 1, sz - 1);
		}

		__device__ __forceinline__ int BrickOfVoxel(int x, int y, int z, const VoxelBricks& vb)
		{
			return x / kVoxelBrick + vb.NX * (y / kVoxelBrick + vb.NY * (z / kVoxelBrick));
		}

		// The ball through the box [lo, hi] of voxel centres, and the margin for rounding.
		__device__ __forceinline__ void BallOf(const float (&lo)[3], const float (&hi)[3], float (&c)[3], float& r, float& margin,
			float scale)
		{
			float e2 = 0.0f;
#pragma unroll
			for (int a = 0; a < 3; ++a)
			{
				c[a] = 0.5f * (lo[a] + hi[a]);
				const float e = 0.5f * (hi[a] - lo[a]);
				e2 += e * e;
			}
			r = sqrtf(e2) * 1.0001f + 1e-6f;
			margin = 1e-4f * (1.0f + fabsf(c[0]) + fabsf(c[1]) + fabsf(c[2]) + scale);
		}

		// One thread per brick of the point cloud's voxels: when the bricks' voxel centres
		// all descend to one octree cell, that cell's program at the ball's centre decides.
		__global__ void __launch_bounds__(128) CloudBricksKernel(DeviceProgram prog, CloudSpec s, VoxelBricks vb,
			uint32_t* __restrict__ brick_bits)
		{
			extern __shared__ float spill[];
			const int b = (int)(blockIdx.x * blockDim.x + threadIdx.x);
			if (b >= vb.NX * vb.NY * vb.NZ) return;
			int lo[3], hi[3];
			BrickRange(b, vb, s.IX, s.IY, s.IZ, lo, hi);
			// Voxel centres float(i) * step + start + half: monotone in i.
			float clo[3], chi[3];
#pragma unroll
			for (int a = 0; a < 3; ++a)
			{
				clo[a] = ((float)lo[a] * s.Step[a] + s.Start[a]) + s.Half[a];
				chi[a] = ((float)hi[a] * s.Step[a] + s.Start[a]) + s.Half[a];
			}
			bool keep = true;
			bool shared;
			const int cell = DescendBox(prog.Nodes, clo[0], chi[0], clo[1], chi[1], clo[2], chi[2], shared);
			const float clip = __ldg(&prog.Nodes[cell].ClipRadius);
			if (shared && clip >= 0.0f && !(__ldg(&prog.Nodes[cell].Flags) & kNodeNoEvaluator))
			{
				float c[3], r, margin;
				BallOf(clo, chi, c, r, margin, fabsf(__ldg(&prog.Nodes[0].ClipRadius)));
				const float px[1] = { c[0] }, py[1] = { c[1] }, pz[1] = { c[2] };
				float f[1];
				RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, f, spill + threadIdx.x, 128);
				keep = !(fabsf(f[0]) > r + s.Diagonal + margin);
			}
			if (keep) atomicOr(brick_bits + (b >> 5), 1u << (b & 31));
		}

		// abs(Octree->Eval(Cursor)) < Diagonal per voxel centre (export.cpp:404-423).
		__global__ void __launch_bounds__(128) CloudFlagsKernel(DeviceProgram prog, CloudSpec s, VoxelBricks vb,
			const uint32_t* __restrict__ brick_bits, uint32_t* __restrict__ words)
		{
			extern __shared__ float spill[];
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool keep = false;
			bool live = false;
			if (t < s.Total)
			{
				const int i = (int)t;
				const int slice = s.IX * s.IY;
				const int b = BrickOfVoxel(i % s.IX, (i % slice) / s.IX, i / slice, vb);
				live = (__ldg(brick_bits + (b >> 5)) >> (b & 31)) & 1u;
			}
			if (live)
			{
				const float d = OctreeDistance(prog, CloudCentre(s, (int)t), spill + threadIdx.x, 128);
				keep = fabsf(d) < s.Diagonal;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, keep);
			if ((threadIdx.x & 31) == 0 && t < s.Total) words[t >> 5] = ballot;
		}

		// SDFOctree::Gradient (the selected cell's SDFNode::Gradient, sdf_evaluator.cpp:298-333)
		// at p: the four tetrahedral evaluations share one pass over the cell's surface
		// program; the evaluation at p itself is needed only when they cancel.
		__device__ __forceinline__ Vec3 OctreeGradient(const DeviceProgram& prog, Vec3 p, float* spill, int stride)
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
			RunSurfaceBatch<4>(prog.Code, pc, px, py, pz, r4, -1, nullptr, spill, stride);
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
				RunSurfaceBatch<1>(prog.Code, pc, qx, qy, qz, r1, -1, nullptr, spill, stride);
				e[4] = r1[0];
			}
			return GradientOf(e);
		}

		// The refinement (export.cpp:434-465): `iterations` steps of Cursor += Gradient *
		// -Eval, clamped to the voxel; the point moves only if it stays within the diagonal.
		// Compiled for 12 resident CTAs per SM (the default took 80 registers, 6 CTAs): the
		// refinement of the 0.01-voxel cloud measured 4.17 ms at 6, 3.85 at 8, 3.58 at 10,
		// 3.47 at 12 and 4.13 at 16.
		__global__ void __launch_bounds__(128, 12) CloudRefineKernel(DeviceProgram prog, CloudSpec s, const uint32_t* __restrict__ cells,
			const uint32_t* __restrict__ count, int iterations, float* __restrict__ points)
		{
			extern __shared__ float spill[];
			const uint32_t n = __ldg(count);
			const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
			if (v >= n) return;
			const Vec3 vertex = CloudCentre(s, (int)__ldg(cells + v));
			const Vec3 half(s.Half[0], s.Half[1], s.Half[2]);
			Vec3 cursor = vertex;
			if (iterations > 0)
			{
				const Vec3 low = vertex - half, high = vertex + half;
				for (int r = 0; r < iterations; ++r)
				{
					const Vec3 dir = OctreeGradient(prog, cursor, spill + threadIdx.x, 128);
					// Octree->Eval(Cursor) * -1.0 rounds back to float exactly: a negation.
					const float dist = -OctreeDistance(prog, cursor, spill + threadIdx.x, 128);
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

		// VoxExport's voxel centre on one axis: mix(Min, Max, (x + .5) / Size), where
		// vec3(x + .5, ...) converts the double sums to float.
		__device__ __forceinline__ float VoxCentre(float lo, float hi, int x, int size)
		{
			return Mix(lo, hi, (float)((double)x + 0.5) / (float)size);
		}

		// One thread per brick of VoxExport's voxels: the whole tree's program at the centre
		// of the ball through the brick's voxel centres decides (a tree with a brush that is
		// not 1-Lipschitz keeps every brick).  mix() rounds each centre separately, so the
		// box is widened by a relative 1e-6 of its coordinates.
		__global__ void __launch_bounds__(128) VoxBricksKernel(DeviceProgram prog, VoxSpec s, VoxelBricks vb,
			uint32_t* __restrict__ brick_bits)
		{
			extern __shared__ float spill[];
			const int b = (int)(blockIdx.x * blockDim.x + threadIdx.x);
			if (b >= vb.NX * vb.NY * vb.NZ) return;
			bool keep = true;
			if (prog.Lipschitz)
			{
				int lo[3], hi[3];
				BrickRange(b, vb, s.SX, s.SY, s.SZ, lo, hi);
				const int size[3] = { s.SX, s.SY, s.SZ };
				float clo[3], chi[3];
#pragma unroll
				for (int a = 0; a < 3; ++a)
				{
					const float u = VoxCentre(s.Min[a], s.Max[a], lo[a], size[a]);
					const float v = VoxCentre(s.Min[a], s.Max[a], hi[a], size[a]);
					const float slack = 1e-6f * (fabsf(u) + fabsf(v) + fabsf(s.Min[a]) + fabsf(s.Max[a]));
					clo[a] = fminf(u, v) - slack;
					chi[a] = fmaxf(u, v) + slack;
				}
				float c[3], r, margin;
				BallOf(clo, chi, c, r, margin, fabsf(__ldg(&prog.Nodes[0].ClipRadius)));
				const float px[1] = { c[0] }, py[1] = { c[1] }, pz[1] = { c[2] };
				float f[1];
				RunSurfaceBatch<1>(prog.Code, prog.FullSurfaceCode, px, py, pz, f, -1, nullptr, spill + threadIdx.x, 128);
				keep = !(fabsf(f[0]) > r + s.Radius + margin);
			}
			if (keep) atomicOr(brick_bits + (b >> 5), 1u << (b & 31));
		}

		// VoxExport's test (magica.cpp:52-64): the voxel centre mix(Min, Max, (x + .5) / Size)
		// on the whole tree (SDFNode::Eval), kept when |d| <= Radius.
		__global__ void __launch_bounds__(128) VoxFlagsKernel(DeviceProgram prog, VoxSpec s, VoxelBricks vb,
			const uint32_t* __restrict__ brick_bits, uint32_t* __restrict__ words)
		{
			extern __shared__ float spill[];
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool keep = false;
			int x = 0, y = 0, z = 0;
			bool live = false;
			if (t < s.Total)
			{
				const int i = (int)t;
				const int slice = s.SX * s.SY;
				z = i / slice; y = (i % slice) / s.SX; x = i % s.SX;
				const int b = BrickOfVoxel(x, y, z, vb);
				live = (__ldg(brick_bits + (b >> 5)) >> (b & 31)) & 1u;
			}
			if (live)
			{
				const float px[1] = { VoxCentre(s.Min[0], s.Max[0], x, s.SX) };
				const float py[1] = { VoxCentre(s.Min[1], s.Max[1], y, s.SY) };
				const float pz[1] = { VoxCentre(s.Min[2], s.Max[2], z, s.SZ) };
				float r[1];
				RunSurfaceBatch<1>(prog.Code, prog.FullSurfaceCode, px, py, pz, r, -1, nullptr, spill + threadIdx.x, 128);
				keep = fabsf(r[0]) <= s.Radius;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, keep);
			if ((threadIdx.x & 31) == 0 && t < s.Total) words[t >> 5] = ballot;
		}
	}

	namespace
	{
		VoxelBricks BricksOf(int sx, int sy, int sz)
		{
			return { (sx + kVoxelBrick - 1) / kVoxelBrick, (sy + kVoxelBrick - 1) / kVoxelBrick, (sz + kVoxelBrick - 1) / kVoxelBrick };
		}

		size_t DistanceSpillBytes(const DeviceProgram& prog, int threads)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			return (size_t)depth * 2 * threads * sizeof(float);
		}
	}

	size_t VoxelBrickWords(int sx, int sy, int sz)
	{
		const VoxelBricks vb = BricksOf(sx, sy, sz);
		return ((size_t)vb.NX * vb.NY * vb.NZ + 31) / 32;
	}

	cudaError_t LaunchCloudFlags(const DeviceProgram& prog, const CloudSpec& s, uint32_t* brick_bits, uint32_t* words, cudaStream_t stream)
	{
		if (s.Total <= 0) return cudaSuccess;
		const VoxelBricks vb = BricksOf(s.IX, s.IY, s.IZ);
		const int nb = vb.NX * vb.NY * vb.NZ;
		cudaError_t e = cudaMemsetAsync(brick_bits, 0, VoxelBrickWords(s.IX, s.IY, s.IZ) * 4, stream);
		if (e != cudaSuccess) return e;
		const size_t smem = DistanceSpillBytes(prog, 128);
		if (smem > 48 * 1024)
		{
			e = cudaFuncSetAttribute(CloudBricksKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e == cudaSuccess) e = cudaFuncSetAttribute(CloudFlagsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		CloudBricksKernel<<<Blocks(nb, 128), 128, smem, stream>>>(prog, s, vb, brick_bits);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		CloudFlagsKernel<<<Blocks(s.Total, 128), 128, smem, stream>>>(prog, s, vb, brick_bits, words);
		return cudaGetLastError();
	}

	cudaError_t LaunchCloudRefine(const DeviceProgram& prog, const CloudSpec& s, const uint32_t* cells, const uint32_t* count,
		uint32_t capacity, int iterations, float* points, cudaStream_t stream)
	{
		if (capacity == 0) return cudaSuccess;
		// The gradient's four-point surface pass: four distances and a material slot per
		// depth (RunSurfaceBatch<4>'s layout), enough for the distance pass too.
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depth * 5 * 128 * sizeof(float);
		if (smem > 48 * 1024)
		{
			const cudaError_t e = cudaFuncSetAttribute(CloudRefineKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		CloudRefineKernel<<<Blocks(capacity, 128), 128, smem, stream>>>(prog, s, cells, count, iterations, points);
		return cudaGetLastError();
	}

	cudaError_t LaunchVoxFlags(const DeviceProgram& prog, const VoxSpec& s, uint32_t* brick_bits, uint32_t* words, cudaStream_t stream)
	{
		if (s.Total <= 0) return cudaSuccess;
		const VoxelBricks vb = BricksOf(s.SX, s.SY, s.SZ);
		const int nb = vb.NX * vb.NY * vb.NZ;
		cudaError_t e = cudaMemsetAsync(brick_bits, 0, VoxelBrickWords(s.SX, s.SY, s.SZ) * 4, stream);
		if (e != cudaSuccess) return e;
		const size_t smem = DistanceSpillBytes(prog, 128);
		if (smem > 48 * 1024)
		{
			e = cudaFuncSetAttribute(VoxFlagsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e == cudaSuccess) e = cudaFuncSetAttribute(VoxBricksKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		VoxBricksKernel<<<Blocks(nb, 128), 128, smem, stream>>>(prog, s, vb, brick_bits);
		e = cudaGetLastError();
		if (e != cudaSuccess) return e;
		VoxFlagsKernel<<<Blocks(s.Total, 128), 128, smem, stream>>>(prog, s, vb, brick_bits, words);
		return cudaGetLastError();
	}
}
