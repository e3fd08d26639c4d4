// Sodapop's meshing job for one drawable (MeshingJob::NaiveSurfaceNets,
// tangerine/sodapop.cpp:562-897) on the GPU.
//
// The reference evaluates the meshing octree with the non-exact descent on a per-axis
// lattice (NaiveSurfaceNetsScratch, sodapop.cpp:150-177), keeps a "point cache" of the
// cell numbers inside the octree's leaves (sodapop.cpp:613-644), runs the surface-nets cell
// pass over the cached cells in increasing order (std::set buckets) and the face pass per
// vertex, then shades every vertex with the gradient and the material's BSDF
// (sodapop.cpp:815-872).  Here the lattice is one kernel, the point cache a byte mask
// written from the leaves' integer boxes, the active cells a bitmask from warp ballots, and
// the vertex numbers a prefix sum over its words, so vertices come out in cell order as
// the serial reference produces them.
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_surface.cuh"

namespace tg
{
	namespace
	{
		inline unsigned Blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

		// SDFOctree::Descend(Point, Exact = false) (sdf_evaluator.cpp:1801-1835): follow the
		// pivot octant to a terminus; a missing child, or a terminus without an evaluator,
		// means no cell (-1: Eval returns +inf).
		__device__ __forceinline__ int DescendLoose(const OctNode* __restrict__ nodes, float x, float y, float z)
		{
			int at = 0;
			for (int guard = 0; guard < 64; ++guard)
			{
				const float4 a = __ldg(reinterpret_cast<const float4*>(nodes + at));
				const int flags = __float_as_int(a.w);
				if (flags & kNodeTerminus) return (flags & kNodeNoEvaluator) ? -1 : at;
				const int octant = (x > a.x ? 1 : 0) | (y > a.y ? 2 : 0) | (z > a.z ? 4 : 0);
				const int child = __ldg(&nodes[at].Child[octant]);
				if (child < 0) return -1;
				at = child;
			}
			return -1;
		}

		// Descend(Point, Exact = true) on an octree that may hold cells without an evaluator:
		// the deepest cell on the point's path that has one (the root always does).
		__device__ __forceinline__ int DescendWithEvaluator(const OctNode* __restrict__ nodes, float x, float y, float z)
		{
			int at = 0, found = 0;
			for (int guard = 0; guard < 64; ++guard)
			{
				const float4 a = __ldg(reinterpret_cast<const float4*>(nodes + at));
				const int flags = __float_as_int(a.w);
				if (!(flags & kNodeNoEvaluator)) found = at;
				if (flags & kNodeTerminus) break;
				const int octant = (x > a.x ? 1 : 0) | (y > a.y ? 2 : 0) | (z > a.z ? 4 : 0);
				const int child = __ldg(&nodes[at].Child[octant]);
				if (child < 0) break;
				at = child;
			}
			return found;
		}

		__device__ __forceinline__ float LatticeAt(const float* __restrict__ lat, const SodapopGrid& g, int64_t i, int64_t j, int64_t k)
		{
			return __ldg(lat + (k * (g.SY + 1) + j) * (g.SX + 1) + i);
		}

		__device__ __forceinline__ void CellOf(const SodapopGrid& g, int64_t c, int64_t& i, int64_t& j, int64_t& k)
		{
			i = c % g.SX;
			j = (c / g.SX) % g.SY;
			k = c / (g.SX * g.SY);
		}

		// Ext.ImplicitFunction (sodapop.cpp:583-587): glm::clamp of the non-exact octree
		// distance to [-100, 100].
		__global__ void __launch_bounds__(128) SodapopLatticeKernel(DeviceProgram prog, SodapopGrid g, float* __restrict__ out, int64_t n)
		{
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (t >= n) return;
			const int64_t nx = g.SX + 1, ny = g.SY + 1;
			const int64_t i = t % nx, j = (t / nx) % ny, k = t / (nx * ny);
			// surface_nets.cpp's grid point: origin + float(index) * step, per axis.
			const float px[1] = { g.G[0] + (float)i * g.D[0] };
			const float py[1] = { g.G[1] + (float)j * g.D[1] };
			const float pz[1] = { g.G[2] + (float)k * g.D[2] };
			float d = __int_as_float(0x7F800000);
			const int cell = DescendLoose(prog.Nodes, px[0], py[0], pz[0]);
			if (cell >= 0)
			{
				float spill[kMaxStack];
				float r[1];
				RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, r, spill, 1);
				d = r[0];
			}
			out[t] = TernaryClamp(d, -100.0f, 100.0f);
		}

		// The point cache (sodapop.cpp:613-644): every number of a leaf's aligned box.  The
		// reference's float loops run over integer values, so the box is integer here; the
		// number wraps into the next row where x passes SX, as the reference's does.
		__global__ void SodapopCacheKernel(const int64_t* __restrict__ boxes, SodapopGrid g, uint8_t* __restrict__ cached)
		{
			const int64_t* b = boxes + (int64_t)blockIdx.x * 6;
			const int64_t x0 = b[0], y0 = b[2], z0 = b[4];
			const int64_t nx = b[1] - x0 + 1, ny = b[3] - y0 + 1, nz = b[5] - z0 + 1;
			if (nx <= 0 || ny <= 0 || nz <= 0) return;
			const int64_t total = nx * ny * nz;
			for (int64_t t = threadIdx.x; t < total; t += blockDim.x)
			{
				const int64_t x = x0 + t % nx, y = y0 + (t / nx) % ny, z = z0 + t / (nx * ny);
				const int64_t n = x + y * g.SX + z * g.SX * g.SY;
				if (n >= 0 && n < g.Limit) cached[n] = 1;
			}
		}

		__global__ void SodapopFlagsKernel(const float* __restrict__ lat, const uint8_t* __restrict__ cached, SodapopGrid g,
			uint32_t* __restrict__ words)
		{
			const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool active = false;
			if (c < g.Limit && __ldg(cached + c))
			{
				int64_t i, j, k;
				CellOf(g, c, i, j, k);
				unsigned pos = 0;
#pragma unroll
				for (int q = 0; q < 8; ++q)
				{
					const float v = LatticeAt(lat, g, i + kCornerOfs[q][0], j + kCornerOfs[q][1], k + kCornerOfs[q][2]);
					pos |= (v >= 0.0f ? 1u : 0u) << q;
				}
				active = pos != 0u && pos != 0xFFu;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
			if ((threadIdx.x & 31) == 0 && c < g.Limit) words[c >> 5] = ballot;
		}

		__device__ __forceinline__ bool Flagged(const SodapopGrid& g, const uint32_t* __restrict__ words, int64_t c)
		{
			return c >= 0 && c < g.Limit && IsActive(words, c);
		}

		// FirstLoopInnerThunk (surface_nets.cpp:864-974): the mean of the bipolar edges'
		// crossings in cell units, mapped to world space per axis; and how many triangles
		// SecondLoopThunk (surface_nets.cpp:1001-1121) will emit for the cell.
		__global__ void SodapopVerticesKernel(const float* __restrict__ lat, SodapopGrid g, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, float* __restrict__ positions, uint32_t* __restrict__ cells,
			uint32_t* __restrict__ face_counts)
		{
			const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (c >= g.Limit) return;
			const uint32_t w = __ldg(words + (c >> 5));
			if (!((w >> (c & 31)) & 1u)) return;
			const uint32_t vid = __ldg(base + (c >> 5)) + __popc(w & ((1u << (c & 31)) - 1u));
			int64_t i, j, k;
			CellOf(g, c, i, j, k);
			float v[8];
#pragma unroll
			for (int q = 0; q < 8; ++q) v[q] = LatticeAt(lat, g, i + kCornerOfs[q][0], j + kCornerOfs[q][1], k + kCornerOfs[q][2]);
			const float fi = (float)i, fj = (float)j, fk = (float)k;
			float sx = 0.0f, sy = 0.0f, sz = 0.0f;
			int count = 0;
#pragma unroll
			for (int e = 0; e < 12; ++e)
			{
				const int a = kEdges[e][0], b = kEdges[e][1];
				const float s1 = v[a], s2 = v[b];
				if ((s1 >= 0.0f) == (s2 >= 0.0f)) continue;
				const float p1x = fi + (float)kCornerOfs[a][0], p1y = fj + (float)kCornerOfs[a][1], p1z = fk + (float)kCornerOfs[a][2];
				const float p2x = fi + (float)kCornerOfs[b][0], p2y = fj + (float)kCornerOfs[b][1], p2z = fk + (float)kCornerOfs[b][2];
				const float t = (0.0f - s1) / (s2 - s1);
				sx = sx + (p1x + t * (p2x - p1x));
				sy = sy + (p1y + t * (p2y - p1y));
				sz = sz + (p1z + t * (p2z - p1z));
				++count;
			}
			const float n = (float)count;
			const float cx = sx / n, cy = sy / n, cz = sz / n;
			const float fsx = (float)g.SX, fsy = (float)g.SY, fsz = (float)g.SZ;
			const float maxx = g.G[0] + fsx * g.D[0], maxy = g.G[1] + fsy * g.D[1], maxz = g.G[2] + fsz * g.D[2];
			positions[(int64_t)vid * 3 + 0] = g.G[0] + (maxx - g.G[0]) * (cx - 0.0f) / (fsx - 0.0f);
			positions[(int64_t)vid * 3 + 1] = g.G[1] + (maxy - g.G[1]) * (cy - 0.0f) / (fsy - 0.0f);
			positions[(int64_t)vid * 3 + 2] = g.G[2] + (maxz - g.G[2]) * (cz - 0.0f) / (fsz - 0.0f);
			cells[vid] = (uint32_t)c;

			uint32_t faces = 0;
			if (i > 0 && j > 0 && k > 0)
			{
				const int64_t dy = g.SX, dz = g.SX * g.SY;
				const bool n0 = Flagged(g, words, c - 1), n1 = Flagged(g, words, c - 1 - dy), n2 = Flagged(g, words, c - dy);
				const bool n3 = Flagged(g, words, c - dy - dz), n4 = Flagged(g, words, c - dz), n5 = Flagged(g, words, c - 1 - dz);
				if (n0 && n1 && n2) faces += 2;
				if (n0 && n5 && n4) faces += 2;
				if (n2 && n3 && n4) faces += 2;
			}
			face_counts[vid] = faces;
		}

		__global__ void SodapopFacesKernel(const float* __restrict__ lat, SodapopGrid g, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, const uint32_t* __restrict__ cells, const uint32_t* __restrict__ face_base,
			uint32_t vertex_count, uint32_t* __restrict__ faces)
		{
			const uint32_t v0 = blockIdx.x * blockDim.x + threadIdx.x;
			if (v0 >= vertex_count) return;
			const int64_t c = __ldg(cells + v0);
			int64_t i, j, k;
			CellOf(g, c, i, j, k);
			if (i == 0 || j == 0 || k == 0) return;
			const int64_t dy = g.SX, dz = g.SX * g.SY;
			const int64_t nb[6] = { c - 1, c - 1 - dy, c - dy, c - dy - dz, c - dz, c - 1 - dz };
			const int quads[3][3] = { {0, 1, 2}, {0, 5, 4}, {2, 3, 4} };
			// The directed edges (0,4), (3,0), (0,1) of the cell decide the winding.
			const float c0 = LatticeAt(lat, g, i, j, k);
			const float s[3][2] = { { c0, LatticeAt(lat, g, i, j, k + 1) }, { LatticeAt(lat, g, i, j + 1, k), c0 },
				{ c0, LatticeAt(lat, g, i + 1, j, k) } };
			uint32_t out = __ldg(face_base + v0);
			for (int q = 0; q < 3; ++q)
			{
				const int64_t a = nb[quads[q][0]], b = nb[quads[q][1]], d = nb[quads[q][2]];
				if (!(Flagged(g, words, a) && Flagged(g, words, b) && Flagged(g, words, d))) continue;
				const uint32_t nv[3] = { VertexOf(words, base, a), VertexOf(words, base, b), VertexOf(words, base, d) };
				uint32_t v1, v2, v3;
				if (s[q][1] > s[q][0]) { v1 = nv[0]; v2 = nv[1]; v3 = nv[2]; }
				else { v1 = nv[2]; v2 = nv[1]; v3 = nv[0]; }
				uint32_t* f = faces + (int64_t)out * 3;
				f[0] = v0; f[1] = v1; f[2] = v2;
				f[3] = v0; f[4] = v2; f[5] = v3;
				out += 2;
			}
		}

		constexpr int kSodaPoints = 32;
		constexpr int kSodaThreads = kSodaPoints * 5;

		// MaterialPBRBR::Eval(P, N, V) with V = N (tangerine/material.cpp:33-40), as the
		// meshing job calls it: D = pow(max(dot(N, H), 0), 2) with H = normalize(N*0.75 + N),
		// F = 1 - max(dot(N, N), 0), colour = RGB * (D + F * 0.25).  The square is one
		// correctly rounded product here; a libm pow(x, 2) may round differently by one ulp.
		__device__ __forceinline__ Vec3 ShadePbr(Vec3 rgb, Vec3 n)
		{
			const Vec3 h = Normalize(n * 0.75f + n);
			const float dd = TernaryMax(Dot(n, h), 0.0f);
			const float D = dd * dd;
			const float F = 1.0f - TernaryMax(Dot(n, n), 0.0f);
			const float bsdf = D + F * 0.25f;
			return rgb * bsdf;
		}

		// Five threads per vertex, as the export's attribute pass: the four tetrahedral
		// evaluations of SDFOctree::Gradient and the point itself for GetMaterial, each on the
		// surface program of the cell the exact descent picks for the vertex.
		__global__ void __launch_bounds__(kSodaThreads) SodapopAttributesKernel(DeviceProgram prog, const float* __restrict__ positions,
			uint32_t n, float* __restrict__ normals, float* __restrict__ colors)
		{
			extern __shared__ float spill[];
			__shared__ float evals[kSodaThreads];
			__shared__ int mats[kSodaPoints];
			const int local = threadIdx.x / 5, lane = threadIdx.x % 5;
			const uint32_t v = blockIdx.x * kSodaPoints + local;
			if (v < n)
			{
				const Vec3 p(positions[(int64_t)v * 3], positions[(int64_t)v * 3 + 1], positions[(int64_t)v * 3 + 2]);
				const int cell = DescendWithEvaluator(prog.Nodes, p.x, p.y, p.z);
				const int pc = __ldg(&prog.Nodes[cell].SurfaceCode);
				const Vec3 q = TetraPoint(p, lane);
				const float px[1] = { q.x }, py[1] = { q.y }, pz[1] = { q.z };
				float e[1];
				int m = -1;
				RunSurfaceBatch<1>(prog.Code, pc, px, py, pz, e, lane == 4 ? 0 : -1, &m, spill + threadIdx.x, kSodaThreads);
				evals[threadIdx.x] = e[0];
				if (lane == 4) mats[local] = m;
			}
			__syncthreads();
			if (v < n && lane == 0)
			{
				const Vec3 g = GradientOf(evals + local * 5);
				normals[(int64_t)v * 3 + 0] = g.x;
				normals[(int64_t)v * 3 + 1] = g.y;
				normals[(int64_t)v * 3 + 2] = g.z;
				const int m = mats[local];
				Vec3 rgb(1.0f, 1.0f, 1.0f);
				if (m >= 0)
				{
					const float4 c = __ldg(prog.MaterialRgb + m);
					rgb = Vec3(c.x, c.y, c.z);
				}
				const Vec3 c = ShadePbr(rgb, g);
				colors[(int64_t)v * 4 + 0] = c.x;
				colors[(int64_t)v * 4 + 1] = c.y;
				colors[(int64_t)v * 4 + 2] = c.z;
				colors[(int64_t)v * 4 + 3] = 1.0f;
			}
		}
	}

	cudaError_t LaunchSodapopLattice(const DeviceProgram& prog, const SodapopGrid& g, float* lattice, cudaStream_t stream)
	{
		const int64_t n = (g.SX + 1) * (g.SY + 1) * g.LZ;
		if (n <= 0) return cudaSuccess;
		SodapopLatticeKernel<<<Blocks(n, 128), 128, 0, stream>>>(prog, g, lattice, n);
		return cudaGetLastError();
	}

	cudaError_t LaunchSodapopCache(const int64_t* boxes, int leaves, const SodapopGrid& g, uint8_t* cached, cudaStream_t stream)
	{
		cudaError_t e = cudaMemsetAsync(cached, 0, (size_t)g.Limit, stream);
		if (e != cudaSuccess || leaves <= 0) return e;
		SodapopCacheKernel<<<(unsigned)leaves, 256, 0, stream>>>(boxes, g, cached);
		return cudaGetLastError();
	}

	cudaError_t LaunchSodapopFlags(const float* lattice, const uint8_t* cached, const SodapopGrid& g, uint32_t* words,
		cudaStream_t stream)
	{
		if (g.Limit <= 0) return cudaSuccess;
		SodapopFlagsKernel<<<Blocks(g.Limit, 256), 256, 0, stream>>>(lattice, cached, g, words);
		return cudaGetLastError();
	}

	cudaError_t LaunchSodapopVertices(const float* lattice, const SodapopGrid& g, const uint32_t* words, const uint32_t* word_base,
		float* positions, uint32_t* cells, uint32_t* face_counts, cudaStream_t stream)
	{
		if (g.Limit <= 0) return cudaSuccess;
		SodapopVerticesKernel<<<Blocks(g.Limit, 256), 256, 0, stream>>>(lattice, g, words, word_base, positions, cells, face_counts);
		return cudaGetLastError();
	}

	cudaError_t LaunchSodapopFaces(const float* lattice, const SodapopGrid& g, const uint32_t* words, const uint32_t* word_base,
		const uint32_t* cells, const uint32_t* face_base, uint32_t vertex_count, uint32_t* faces, cudaStream_t stream)
	{
		if (vertex_count == 0) return cudaSuccess;
		SodapopFacesKernel<<<Blocks(vertex_count, 256), 256, 0, stream>>>(lattice, g, words, word_base, cells, face_base, vertex_count,
			faces);
		return cudaGetLastError();
	}

	cudaError_t LaunchSodapopAttributes(const DeviceProgram& prog, const float* positions, uint32_t vertex_count, float* normals,
		float* colors, cudaStream_t stream)
	{
		if (vertex_count == 0) return cudaSuccess;
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depth * 2 * kSodaThreads * sizeof(float);
		if (smem > 40 * 1024)
		{
			cudaError_t e = cudaFuncSetAttribute(SodapopAttributesKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		SodapopAttributesKernel<<<Blocks(vertex_count, kSodaPoints), kSodaThreads, smem, stream>>>(prog, positions, vertex_count, normals,
			colors);
		return cudaGetLastError();
	}
}
