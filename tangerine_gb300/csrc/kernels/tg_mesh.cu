// Naive surface nets over an evaluated lattice, and per-vertex normals and colours.
//
// The reference (third_party/naive-surface-nets/src/surface_nets.cpp:829-1122) pushes a
// vertex per active cell under a mutex and keeps an unordered_map from cube index to
// vertex.  Here the active cells become a bitmask built from warp ballots; a prefix sum
// over the words' popcounts gives every active cell its vertex number, in cell order, which
// is the order the reference's serial pstl backend produces.  A neighbour's vertex is the
// popcount-rank lookup in that bitmask, so no map is built.
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_surface.cuh"
#include "tg_pair.cuh"

namespace tg
{
	namespace
	{
		__global__ void CellFlagsKernel(const float* __restrict__ lat, GridSpec g, uint32_t* __restrict__ words, int64_t cells)
		{
			const CellGeom cg = Geom(g);
			const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool active = false;
			if (c < cells)
			{
				const int64_t i = c % cg.sx;
				const int64_t j = (c / cg.sx) % cg.sy;
				const int64_t k = c / (cg.sx * cg.sy);
				float v[8];
				LoadCorners(lat, cg, i, j, k, v);
				// "Positive" is >= isovalue (0); a cell with two signs has a bipolar edge.
				unsigned pos = 0;
#pragma unroll
				for (int q = 0; q < 8; ++q) pos |= (v[q] >= 0.0f ? 1u : 0u) << q;
				active = pos != 0u && pos != 0xFFu;
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
			if ((threadIdx.x & 31) == 0 && c < cells) words[c >> 5] = ballot;
		}

		__global__ void CellVerticesKernel(const float* __restrict__ lat, GridSpec g, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, float* __restrict__ vertices, uint32_t* __restrict__ cubes,
			uint32_t* __restrict__ face_counts, int64_t cells)
		{
			const CellGeom cg = Geom(g);
			const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (c >= cells) return;
			const uint32_t w = __ldg(words + (c >> 5));
			if (!((w >> (c & 31)) & 1u)) return;
			const uint32_t vid = __ldg(base + (c >> 5)) + __popc(w & ((1u << (c & 31)) - 1u));
			const int64_t i = c % cg.sx;
			const int64_t j = (c / cg.sx) % cg.sy;
			const int64_t k = c / (cg.sx * cg.sy);
			EmitCellVertex(lat, g, cg, words, c, i, j, k, vid, vertices, cubes, face_counts);
		}

		__global__ void FacesKernel(const float* __restrict__ lat, GridSpec g, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, const uint32_t* __restrict__ cubes, const uint32_t* __restrict__ face_base,
			uint32_t vertex_count, uint32_t* __restrict__ faces)
		{
			const CellGeom cg = Geom(g);
			const uint32_t v0 = blockIdx.x * blockDim.x + threadIdx.x;
			if (v0 >= vertex_count) return;
			const int64_t c = __ldg(cubes + v0);
			const int64_t i = c % cg.sx;
			const int64_t j = (c / cg.sx) % cg.sy;
			const int64_t k = c / (cg.sx * cg.sy);
			if (i == 0 || j == 0 || k == 0) return;
			const int64_t dy = cg.sx, dz = cg.sx * cg.sy;
			const int64_t nb[6] = { c - 1, c - 1 - dy, c - dy, c - dy - dz, c - dz, c - 1 - dz };
			const int quads[3][3] = { {0, 1, 2}, {0, 5, 4}, {2, 3, 4} };
			// Directed edges (0,4), (3,0), (0,1) decide the winding (surface_nets.cpp:1041-1105).
			const float c0 = Corner(lat, cg, i, j, k);
			const float s[3][2] = { { c0, Corner(lat, cg, i, j, k + 1) }, { Corner(lat, cg, i, j + 1, k), c0 }, { c0, Corner(lat, cg, i + 1, j, k) } };
			uint32_t out = __ldg(face_base + v0);
			for (int q = 0; q < 3; ++q)
			{
				const int64_t a = nb[quads[q][0]], b = nb[quads[q][1]], d = nb[quads[q][2]];
				if (!(IsActive(words, a) && IsActive(words, b) && IsActive(words, d))) continue;
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

		// Face normals (the STL writer): five threads per point (the four tetrahedral offsets
		// of SDFNode::Gradient and the point itself), each a single pass over the point's
		// surface program; lane 0 combines them.  One lane per evaluation keeps the
		// interpreter's code small enough for the instruction cache.
		constexpr int kPointsPerBlock = 32;
		constexpr int kAttribThreads = kPointsPerBlock * 5;

		// One evaluation lane: distance at TetraPoint(p, lane); lane 4 with `material` also
		// returns the material index.  `stride`: the block's thread count (spill layout).
		__device__ __forceinline__ float EvaluationLane(const DeviceProgram& prog, Vec3 p, int lane, bool material, int* m, float* spill,
			int stride = kAttribThreads)
		{
			const int cell = DescendOctree(prog.Nodes, p.x, p.y, p.z);
			const int pc = __ldg(&prog.Nodes[cell].SurfaceCode);
			const Vec3 q = TetraPoint(p, lane);
			const float px[1] = { q.x }, py[1] = { q.y }, pz[1] = { q.z };
			float e[1];
			RunSurfaceBatch<1>(prog.Code, pc, px, py, pz, e, (lane == 4 && material) ? 0 : -1, m, spill, stride);
			return e[0];
		}

		// Normals alone: two threads per vertex, each evaluating two of the four tetrahedral
		// points as one pair (tg_pair.cuh), all running the same code; lane 0 combines them and
		// evaluates the vertex itself only when the four cancel (SDFNode::Gradient's
		// fallback).  The colours are a separate pass, so no lane takes the material path
		// while the others wait.
		constexpr int kNormalThreads = 128;
		constexpr int kNormalPoints = kNormalThreads / 2;

		// The vertex the attribute passes visit at position t (VertexOrder in tg_kernels.hpp).
		__device__ __forceinline__ uint32_t VertexAt(const VertexOrder& o, uint32_t t)
		{
			if (!o.Cells) return t;
			const uint32_t c = __ldg(o.Cells + t);
			const uint32_t w = __ldg(o.Words + (c >> 5));
			return __ldg(o.Base + (c >> 5)) + __popc(w & ((1u << (c & 31)) - 1u));
		}

		__global__ void __launch_bounds__(kNormalThreads) VertexNormalsKernel(DeviceProgram prog, const float* __restrict__ vertices,
			uint32_t n, float* __restrict__ normals, VertexOrder order)
		{
			extern __shared__ float spill[];
			const int local = threadIdx.x >> 1, lane = threadIdx.x & 1;
			const uint32_t t = blockIdx.x * kNormalPoints + local;
			const uint32_t v = t < n ? VertexAt(order, t) : n;
			Vec3 p(0.0f, 0.0f, 0.0f);
			float2 mine = make_float2(0.0f, 0.0f);
			int pc = 0;
			const float4* code = prog.Code;
			auto load = [&](int q) { return __ldg(code + q); };
			float2* spill2 = reinterpret_cast<float2*>(spill) + threadIdx.x;
			if (v < n)
			{
				p = Vec3(vertices[(int64_t)v * 3], vertices[(int64_t)v * 3 + 1], vertices[(int64_t)v * 3 + 2]);
				const int cell = DescendOctree(prog.Nodes, p.x, p.y, p.z);
				pc = __ldg(&prog.Nodes[cell].SurfaceCode);
				const Vec3 a = TetraPoint(p, 2 * lane), b = TetraPoint(p, 2 * lane + 1);
				mine = RunSurfacePair(load, pc, make_float2(a.x, b.x), make_float2(a.y, b.y), make_float2(a.z, b.z), spill2,
					kNormalThreads);
			}
			// The two lanes of a vertex are neighbours in one warp.
			const int first = (threadIdx.x & 31) & ~1;
			float e[5];
			e[0] = __shfl_sync(0xFFFFFFFFu, mine.x, first);
			e[1] = __shfl_sync(0xFFFFFFFFu, mine.y, first);
			e[2] = __shfl_sync(0xFFFFFFFFu, mine.x, first + 1);
			e[3] = __shfl_sync(0xFFFFFFFFu, mine.y, first + 1);
			if (v < n && lane == 0)
			{
				e[4] = 0.0f;
				const float h = 0.0001f;
				const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
				Vec3 g = xyy * e[0];
				g = g + yyx * e[1];
				g = g + yxy * e[2];
				g = g + xxx * e[3];
				if ((g.x * g.x + g.y * g.y) + g.z * g.z == 0.0f)
				{
					// The vertex itself, in the same spill layout (both lanes of the pair at p).
					e[4] = RunSurfacePair(load, pc, make_float2(p.x, p.x), make_float2(p.y, p.y), make_float2(p.z, p.z), spill2,
						kNormalThreads).x;
				}
				const Vec3 r = GradientOf(e);
				normals[(int64_t)v * 3 + 0] = r.x;
				normals[(int64_t)v * 3 + 1] = r.y;
				normals[(int64_t)v * 3 + 2] = r.z;
			}
		}

		// Colours: GetMaterial's walk at each vertex, one thread per vertex.
		constexpr int kColorThreads = 128;

		__global__ void __launch_bounds__(kColorThreads) VertexColorsKernel(DeviceProgram prog, const float* __restrict__ vertices,
			uint32_t n, uint8_t* __restrict__ colors, VertexOrder order)
		{
			extern __shared__ float spill[];
			const uint32_t t = blockIdx.x * kColorThreads + threadIdx.x;
			if (t >= n) return;
			const uint32_t v = VertexAt(order, t);
			const Vec3 p(vertices[(int64_t)v * 3], vertices[(int64_t)v * 3 + 1], vertices[(int64_t)v * 3 + 2]);
			int m = -1;
			EvaluationLane(prog, p, 4, true, &m, spill + threadIdx.x, kColorThreads);
			const uchar4 c = m >= 0 ? prog.Colors[m] : make_uchar4(255, 255, 255, 255);
			colors[(int64_t)v * 3 + 0] = c.x;
			colors[(int64_t)v * 3 + 1] = c.y;
			colors[(int64_t)v * 3 + 2] = c.z;
		}

		// WriteSTL(Octree, ...) (export.cpp:140-148): the gradient at (a + b + c) / 3.
		__global__ void __launch_bounds__(kAttribThreads) FaceNormalsKernel(DeviceProgram prog, const float* __restrict__ vertices,
			const uint32_t* __restrict__ faces, uint64_t n, float* __restrict__ normals)
		{
			extern __shared__ float spill[];
			__shared__ float evals[kAttribThreads];
			const int local = threadIdx.x / 5, lane = threadIdx.x % 5;
			const uint64_t f = (uint64_t)blockIdx.x * kPointsPerBlock + local;
			if (f < n)
			{
				const uint32_t a = faces[f * 3], b = faces[f * 3 + 1], c = faces[f * 3 + 2];
				const Vec3 va(vertices[(int64_t)a * 3], vertices[(int64_t)a * 3 + 1], vertices[(int64_t)a * 3 + 2]);
				const Vec3 vb(vertices[(int64_t)b * 3], vertices[(int64_t)b * 3 + 1], vertices[(int64_t)b * 3 + 2]);
				const Vec3 vc(vertices[(int64_t)c * 3], vertices[(int64_t)c * 3 + 1], vertices[(int64_t)c * 3 + 2]);
				const Vec3 s = (va + vb) + vc;
				const Vec3 center(s.x / 3.0f, s.y / 3.0f, s.z / 3.0f);
				evals[threadIdx.x] = EvaluationLane(prog, center, lane, false, nullptr, spill + threadIdx.x);
			}
			__syncthreads();
			if (f < n && lane == 0)
			{
				const Vec3 g = GradientOf(evals + local * 5);
				normals[f * 3] = g.x;
				normals[f * 3 + 1] = g.y;
				normals[f * 3 + 2] = g.z;
			}
		}

		__global__ void EvalPointsKernel(DeviceProgram prog, const float* __restrict__ points, int64_t n, float* __restrict__ out)
		{
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (t >= n) return;
			float spill[kMaxStack];
			const float px[1] = { points[t * 3] }, py[1] = { points[t * 3 + 1] }, pz[1] = { points[t * 3 + 2] };
			float r[1];
			const int cell = DescendOctree(prog.Nodes, px[0], py[0], pz[0]);
			RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, r, spill, 1);
			out[t] = r[0];
		}

		// ---- exclusive scan: 1024 threads x 4 items per block -------------------------
		constexpr int kScanThreads = 1024;
		constexpr int kScanItems = 4;
		constexpr int kScanTile = kScanThreads * kScanItems;

		__device__ __forceinline__ uint32_t ScanItem(const uint32_t* in, int64_t i, int64_t n, bool pop)
		{
			if (i >= n) return 0u;
			const uint32_t x = __ldg(in + i);
			return pop ? (uint32_t)__popc(x) : x;
		}

		// Block-wide exclusive scan of one value per thread; returns the block total.
		__device__ __forceinline__ uint32_t BlockExclusiveScan(uint32_t x, uint32_t& exclusive)
		{
			__shared__ uint32_t warpSums[32];
			const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
			uint32_t inc = x;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1)
			{
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
				if (lane >= o) inc += y;
			}
			if (lane == 31) warpSums[warp] = inc;
			__syncthreads();
			if (warp == 0)
			{
				const uint32_t s = lane < (int)(blockDim.x >> 5) ? warpSums[lane] : 0u;
				uint32_t si = s;
#pragma unroll
				for (int o = 1; o < 32; o <<= 1)
				{
					const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, si, o);
					if (lane >= o) si += y;
				}
				warpSums[lane] = si - s;
			}
			__syncthreads();
			exclusive = warpSums[warp] + inc - x;
			uint32_t total = 0;
			if (threadIdx.x == blockDim.x - 1) total = exclusive + x;
			__syncthreads();
			return total;   // valid in the last thread only
		}

		__global__ void __launch_bounds__(kScanThreads) ScanReduceKernel(const uint32_t* __restrict__ in, int64_t n, bool pop, uint32_t* __restrict__ sums)
		{
			const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
			uint32_t s = 0;
#pragma unroll
			for (int q = 0; q < kScanItems; ++q) s += ScanItem(in, base + q, n, pop);
			uint32_t ex;
			const uint32_t total = BlockExclusiveScan(s, ex);
			if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = total;
		}

		__global__ void __launch_bounds__(kScanThreads) ScanTopKernel(uint32_t* __restrict__ sums, int64_t nb, uint32_t* __restrict__ total)
		{
			__shared__ uint32_t carry;
			if (threadIdx.x == 0) carry = 0;
			__syncthreads();
			for (int64_t start = 0; start < nb; start += kScanThreads)
			{
				const int64_t i = start + threadIdx.x;
				const uint32_t x = i < nb ? sums[i] : 0u;
				uint32_t ex;
				const uint32_t t = BlockExclusiveScan(x, ex);
				const uint32_t c = carry;
				if (i < nb) sums[i] = c + ex;
				__syncthreads();
				if (threadIdx.x == kScanThreads - 1) carry = c + t;
				__syncthreads();
			}
			if (threadIdx.x == 0) *total = carry;
		}

		__global__ void __launch_bounds__(kScanThreads) ScanDownKernel(const uint32_t* __restrict__ in, int64_t n, bool pop,
			const uint32_t* __restrict__ offsets, uint32_t* __restrict__ out)
		{
			const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
			uint32_t v[kScanItems];
			uint32_t s = 0;
#pragma unroll
			for (int q = 0; q < kScanItems; ++q) { v[q] = ScanItem(in, base + q, n, pop); s += v[q]; }
			uint32_t ex;
			BlockExclusiveScan(s, ex);
			uint32_t run = __ldg(offsets + blockIdx.x) + ex;
#pragma unroll
			for (int q = 0; q < kScanItems; ++q)
			{
				if (base + q < n) out[base + q] = run;
				run += v[q];
			}
		}

		inline unsigned Blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }
	}

	size_t ScanScratchWords(int64_t n)
	{
		return (size_t)((n + kScanTile - 1) / kScanTile) + 1;
	}

	cudaError_t LaunchExclusiveScan(const uint32_t* in, int64_t n, bool popcount, uint32_t* out, uint32_t* total,
		uint32_t* scratch, cudaStream_t stream)
	{
		const int64_t nb = (n + kScanTile - 1) / kScanTile;
		if (nb == 0)
		{
			return cudaMemsetAsync(total, 0, sizeof(uint32_t), stream);
		}
		ScanReduceKernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(in, n, popcount, scratch);
		ScanTopKernel<<<1, kScanThreads, 0, stream>>>(scratch, nb, total);
		ScanDownKernel<<<(unsigned)nb, kScanThreads, 0, stream>>>(in, n, popcount, scratch, out);
		return cudaGetLastError();
	}

	cudaError_t LaunchCellFlags(const float* lattice, const GridSpec& grid, uint32_t* words, cudaStream_t stream)
	{
		const int64_t cells = (int64_t)(grid.NX - 1) * (grid.NY - 1) * (grid.NZ - 1);
		if (cells <= 0) return cudaSuccess;
		CellFlagsKernel<<<Blocks(cells, 256), 256, 0, stream>>>(lattice, grid, words, cells);
		return cudaGetLastError();
	}

	cudaError_t LaunchCellVertices(const float* lattice, const GridSpec& grid, const uint32_t* words, const uint32_t* word_base,
		float* vertices, uint32_t* cubes, uint32_t* face_counts, int64_t cells, cudaStream_t stream)
	{
		if (cells <= 0) return cudaSuccess;
		CellVerticesKernel<<<Blocks(cells, 256), 256, 0, stream>>>(lattice, grid, words, word_base, vertices, cubes, face_counts, cells);
		return cudaGetLastError();
	}

	cudaError_t LaunchFaces(const float* lattice, const GridSpec& grid, const uint32_t* words, const uint32_t* word_base,
		const uint32_t* cubes, const uint32_t* face_base, uint32_t vertex_count, uint32_t* faces, cudaStream_t stream)
	{
		if (vertex_count == 0) return cudaSuccess;
		FacesKernel<<<Blocks(vertex_count, 256), 256, 0, stream>>>(lattice, grid, words, word_base, cubes, face_base, vertex_count, faces);
		return cudaGetLastError();
	}

	cudaError_t LaunchEvalPoints(const DeviceProgram& prog, const float* points, int64_t n, float* out, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		EvalPointsKernel<<<Blocks(n, 128), 128, 0, stream>>>(prog, points, n, out);
		return cudaGetLastError();
	}

	// Shared memory of the single-lane surface evaluation: distance + material per level.
	static size_t SurfaceSpillBytes(const DeviceProgram& prog, int threads)
	{
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		return (size_t)depth * 2 * threads * sizeof(float);
	}

	cudaError_t LaunchFaceNormals(const DeviceProgram& prog, const float* vertices, const uint32_t* faces, uint64_t face_count,
		float* normals, cudaStream_t stream)
	{
		if (face_count == 0) return cudaSuccess;
		const size_t smem = SurfaceSpillBytes(prog, kAttribThreads);
		if (smem > 40 * 1024) cudaFuncSetAttribute(FaceNormalsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		FaceNormalsKernel<<<Blocks((int64_t)face_count, kPointsPerBlock), kAttribThreads, smem, stream>>>(prog, vertices, faces,
			face_count, normals);
		return cudaGetLastError();
	}

	cudaError_t LaunchVertexAttributes(const DeviceProgram& prog, const float* vertices, uint32_t vertex_count,
		float* normals, uint8_t* colors, cudaStream_t stream, VertexOrder order)
	{
		if (vertex_count == 0) return cudaSuccess;
		const size_t smem = SurfaceSpillBytes(prog, kNormalThreads);
		if (smem > 40 * 1024) cudaFuncSetAttribute(VertexNormalsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		VertexNormalsKernel<<<Blocks(vertex_count, kNormalPoints), kNormalThreads, smem, stream>>>(prog, vertices, vertex_count, normals,
			order);
		cudaError_t e = cudaGetLastError();
		if (e != cudaSuccess || !colors) return e;
		const size_t csmem = SurfaceSpillBytes(prog, kColorThreads);
		if (csmem > 40 * 1024) cudaFuncSetAttribute(VertexColorsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem);
		VertexColorsKernel<<<Blocks(vertex_count, kColorThreads), kColorThreads, csmem, stream>>>(prog, vertices, vertex_count, colors,
			order);
		return cudaGetLastError();
	}
}
