// Exact brick culling for the mesh export.
//
// The lattice's cells are grouped into bricks of B^3 cells.  A brick can be skipped when
// the distance field provably keeps one sign over it: take the octree cell whose clip
// sphere holds the brick's bounding ball with room to spare, evaluate that cell's clipped
// program at the ball's centre, and compare |f| with the ball's radius.  Every primitive
// here except the ellipsoid estimate is 1-Lipschitz, and union/inter/diff, the polynomial
// blends, flate and uniform scale keep that, so |f(c)| > r + margin means no sign change
// inside the ball.  Inside a cell's clip sphere (shrunk by the margin) the clipped program
// has the sign of the full tree, and so does every other cell's program at its own
// samples: the reference's distances at the brick's samples therefore share one sign and
// the brick holds no active cell.  Skipped bricks produce exactly what the dense path
// produces there -- nothing -- so the mesh is unchanged bit for bit.
//
// The surviving bricks are compacted with warp ballots into a list; a persistent grid
// evaluates the (B+1)^3 lattice points of each listed brick; the cell pass then treats
// cells of skipped bricks as inactive without reading their corners.
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_surface.cuh"

namespace tg
{
	namespace
	{
		constexpr int kClassifyThreads = 128;
		constexpr int kBrickThreads = 128;     // 8 x 8 columns x 2 z-groups of 4 points

		struct BrickGrid
		{
			int B;                  // cells per brick edge
			int NBX, NBY, NBZ;      // bricks per axis
		};

		// Whether the lattice box [i0, i1] x [j0, j1] x [k0, k1] (corner indices) may hold a
		// sign change of the reference's distances; false only when that is proven.
		__device__ __forceinline__ bool BoxMayHoldSurface(const DeviceProgram& prog, const GridSpec& g,
			int i0, int i1, int j0, int j1, int k0, int k1, float* spill, int stride)
		{
			const float x0 = LatticeCoord(g.X0, i0, g.Step), x1 = LatticeCoord(g.X0, i1, g.Step);
			const float y0 = LatticeCoord(g.Y0, j0, g.Step), y1 = LatticeCoord(g.Y0, j1, g.Step);
			const float z0 = LatticeCoord(g.Z0, k0, g.Step), z1 = LatticeCoord(g.Z0, k1, g.Step);
			const float cx = 0.5f * (x0 + x1), cy = 0.5f * (y0 + y1), cz = 0.5f * (z0 + z1);
			const float ex = 0.5f * (x1 - x0), ey = 0.5f * (y1 - y0), ez = 0.5f * (z1 - z0);
			// Ball through the box's corners, widened for the rounding of the centre.
			const float r = sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f + 1e-6f;
			const float rootClip = __ldg(&prog.Nodes[0].ClipRadius);
			const float margin = 1e-4f * (1.0f + fabsf(cx) + fabsf(cy) + fabsf(cz) + fabsf(rootClip));
			// Outside the root cube every brush, and so every clipped program, is positive
			// (the cube holds the tree's bounds): a ball missing the cube has no surface.
			const float half = fabsf(rootClip) * 0.57736f;           // span / 2 = radius / sqrt(3), rounded up
			const float ox = fmaxf(fabsf(cx - __ldg(&prog.Nodes[0].Pivot[0])) - half, 0.0f);
			const float oy = fmaxf(fabsf(cy - __ldg(&prog.Nodes[0].Pivot[1])) - half, 0.0f);
			const float oz = fmaxf(fabsf(cz - __ldg(&prog.Nodes[0].Pivot[2])) - half, 0.0f);
			if (sqrtf(ox * ox + oy * oy + oz * oz) > r + margin) return false;
			// Deepest cell on the centre's descent path whose clip sphere holds the ball.
			int path[48];
			int depth = 0;
			int at = 0;
			path[depth++] = 0;
			for (int guard = 0; guard < 47; ++guard)
			{
				const OctNode* n = prog.Nodes + at;
				const int32_t flags = __ldg(&n->Flags);
				if (flags & kNodeTerminus) break;
				const float px = __ldg(&n->Pivot[0]), py = __ldg(&n->Pivot[1]), pz = __ldg(&n->Pivot[2]);
				const int octant = (cx > px ? 1 : 0) | (cy > py ? 2 : 0) | (cz > pz ? 4 : 0);
				const int child = __ldg(&n->Child[octant]);
				if (child < 0)
				{
					// The octree dropped this octant because its clip returned null: the parent's
					// program exceeds the octant sphere's radius at its centre, so (1-Lipschitz) it
					// stays above the margin inside that sphere shrunk by the margin.  The octant
					// sphere sits inside the parent's, where the parent's program has the tree's
					// sign.  (Octants dropped because all their own children clipped away prove
					// only their cube, without margin, and are not used.)
					const float clip = __ldg(&n->ClipRadius);
					if (clip > 0.0f && ((flags >> (8 + octant)) & 1))
					{
						const float q = clip * 0.28867513f;               // span / 4 = radius / (2 sqrt 3)
						const float qx = px + ((octant & 1) ? q : -q), qy = py + ((octant & 2) ? q : -q), qz = pz + ((octant & 4) ? q : -q);
						const float dx = cx - qx, dy = cy - qy, dz = cz - qz;
						if (sqrtf(dx * dx + dy * dy + dz * dz) + r + margin <= clip * 0.4999f) return false;
					}
					break;
				}
				at = child;
				path[depth++] = at;
			}
			int holder = -1;
			for (int d = depth - 1; d >= 0; --d)
			{
				const OctNode* n = prog.Nodes + path[d];
				const float clip = __ldg(&n->ClipRadius);
				if (clip < 0.0f) break;                           // not 1-Lipschitz here or above
				const float dx = cx - __ldg(&n->Pivot[0]), dy = cy - __ldg(&n->Pivot[1]), dz = cz - __ldg(&n->Pivot[2]);
				if (sqrtf(dx * dx + dy * dy + dz * dz) + r + margin <= clip) { holder = path[d]; break; }
			}
			if (holder < 0) return true;
			const float px[1] = { cx }, py[1] = { cy }, pz[1] = { cz };
			float f[1];
			RunDistance<1>(prog.Code, __ldg(&prog.Nodes[holder].DistanceCode), px, py, pz, f, spill, stride);
			return !(fabsf(f[0]) > r + margin);
		}

		__global__ void __launch_bounds__(kClassifyThreads) ClassifyBricksKernel(DeviceProgram prog, GridSpec g, BrickGrid bg,
			uint32_t* __restrict__ brick_bits, uint32_t* __restrict__ list, uint32_t* __restrict__ count)
		{
			extern __shared__ float spill[];
			const int64_t nb = (int64_t)bg.NBX * bg.NBY * bg.NBZ;
			const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool active = false;
			if (b < nb)
			{
				const int bx = (int)(b % bg.NBX), by = (int)((b / bg.NBX) % bg.NBY), bz = (int)(b / ((int64_t)bg.NBX * bg.NBY));
				const int sx = g.NX - 1, sy = g.NY - 1, sz = g.NZ - 1;
				const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
				active = BoxMayHoldSurface(prog, g, i0, min(i0 + bg.B, sx), j0, min(j0 + bg.B, sy), k0, min(k0 + bg.B, sz),
					spill + threadIdx.x, kClassifyThreads);
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
			const int lane = threadIdx.x & 31;
			if (lane == 0 && b < nb) brick_bits[b >> 5] = ballot;
			uint32_t base = 0;
			if (lane == 0 && ballot) base = atomicAdd(count, (uint32_t)__popc(ballot));
			base = __shfl_sync(0xFFFFFFFFu, base, 0);
			if (active) list[base + __popc(ballot & ((1u << lane) - 1u))] = (uint32_t)b;
		}

		// Lattice points of every listed brick: corners [i0, i0 + B] per axis, clamped to the
		// lattice.  A CTA takes bricks from the list with a grid stride; each thread runs
		// four z-consecutive points through one pass over their octree cell's records.
		// A CTA is 8 x 8 columns x (128 / 64) z-groups; each thread runs K z-consecutive
		// points, so one pass covers an 8 x 8 x 2K chunk of the brick's lattice box.
		template<int C, int K>
		__global__ void __launch_bounds__(kBrickThreads) EvalBricksKernel(DeviceProgram prog, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, float* __restrict__ lattice)
		{
			extern __shared__ float spill[];
			constexpr int ZSpan = 2 * K;
			const uint32_t n = *count;
			const int tx = threadIdx.x & 7, ty = (threadIdx.x >> 3) & 7, tz = threadIdx.x >> 6;
			for (uint32_t item = blockIdx.x; item < n; item += gridDim.x)
			{
				const uint32_t b = __ldg(list + item);
				const int bx = (int)(b % (uint32_t)bg.NBX), by = (int)((b / (uint32_t)bg.NBX) % (uint32_t)bg.NBY);
				const int bz = (int)(b / ((uint32_t)bg.NBX * (uint32_t)bg.NBY));
				const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
				const int i1 = min(i0 + bg.B, g.NX - 1), j1 = min(j0 + bg.B, g.NY - 1), k1 = min(k0 + bg.B, g.NZ - 1);
				for (int oz = 0; oz < C; oz += ZSpan)
				for (int oy = 0; oy < C; oy += 8)
				for (int ox = 0; ox < C; ox += 8)
				{
					const int ix = i0 + ox + tx, iy = j0 + oy + ty, izb = k0 + oz + tz * K;
					const bool inPlane = ix <= i1 && iy <= j1;
					const float x = LatticeCoord(g.X0, min(ix, i1), g.Step);
					const float y = LatticeCoord(g.Y0, min(iy, j1), g.Step);
					float px[K], py[K], pz[K], res[K];
					int cell[K];
					unsigned todo = 0;
#pragma unroll
					for (int k = 0; k < K; ++k)
					{
						const int iz = izb + k;
						px[k] = x;
						py[k] = y;
						pz[k] = LatticeCoord(g.Z0, min(iz, k1), g.Step);
						cell[k] = DescendOctree(prog.Nodes, px[k], py[k], pz[k]);
						res[k] = 0.0f;
						if (inPlane && iz <= k1) todo |= 1u << k;
					}
					while (todo)
					{
						int c = -1;
#pragma unroll
						for (int k = 0; k < K; ++k)
							if (c < 0 && ((todo >> k) & 1u)) c = cell[k];
						float r[K];
						RunDistance<K>(prog.Code, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r, spill + threadIdx.x, kBrickThreads);
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
							const int iz = izb + k;
							if (iz <= k1) lattice[((int64_t)iz * g.NY + iy) * g.NX + ix] = res[k];
						}
					}
				}
			}
		}

		// Cell pass over the lattice of listed bricks only: cells of skipped bricks are
		// inactive without looking at their corners.
		__global__ void CellFlagsBricksKernel(const float* __restrict__ lat, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ brick_bits, uint32_t* __restrict__ words, int64_t cells)
		{
			const int64_t sx = g.NX - 1, sy = g.NY - 1;
			const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			bool active = false;
			if (c < cells)
			{
				const int64_t i = c % sx;
				const int64_t j = (c / sx) % sy;
				const int64_t k = c / (sx * sy);
				const int64_t brick = (i / bg.B) + (int64_t)bg.NBX * ((j / bg.B) + (int64_t)bg.NBY * (k / bg.B));
				if ((__ldg(brick_bits + (brick >> 5)) >> (brick & 31)) & 1u)
				{
					const int64_t nx = g.NX, ny = g.NY;
					const int64_t base = (k * ny + j) * nx + i;
					const int64_t dy = nx, dz = nx * ny;
					const float v[8] = { __ldg(lat + base), __ldg(lat + base + 1), __ldg(lat + base + dy + 1), __ldg(lat + base + dy),
						__ldg(lat + base + dz), __ldg(lat + base + dz + 1), __ldg(lat + base + dz + dy + 1), __ldg(lat + base + dz + dy) };
					unsigned pos = 0;
#pragma unroll
					for (int q = 0; q < 8; ++q) pos |= (v[q] >= 0.0f ? 1u : 0u) << q;
					active = pos != 0u && pos != 0xFFu;
				}
			}
			const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
			if ((threadIdx.x & 31) == 0 && c < cells) words[c >> 5] = ballot;
		}

		// The cells of listed bricks, a CTA per brick with a grid stride over the list.
		// Cells of unlisted bricks hold no surface and are never visited: the active-cell
		// bitmask starts zeroed and only listed cells can set their bit.
		struct BrickCells
		{
			int64_t i0, j0, k0;
			int nx, ny, nz;
		};

		__device__ __forceinline__ BrickCells CellsOf(uint32_t b, const BrickGrid& bg, const CellGeom& cg)
		{
			const int bx = (int)(b % (uint32_t)bg.NBX), by = (int)((b / (uint32_t)bg.NBX) % (uint32_t)bg.NBY);
			const int bz = (int)(b / ((uint32_t)bg.NBX * (uint32_t)bg.NBY));
			BrickCells bc;
			bc.i0 = (int64_t)bx * bg.B; bc.j0 = (int64_t)by * bg.B; bc.k0 = (int64_t)bz * bg.B;
			bc.nx = (int)min((int64_t)bg.B, cg.sx - bc.i0);
			bc.ny = (int)min((int64_t)bg.B, cg.sy - bc.j0);
			bc.nz = (int)min((int64_t)bg.B, cg.sz - bc.k0);
			return bc;
		}

		// Also appends each active cell's index to `cells` (in no particular order: vertex
		// numbers come from the bitmask rank, which is independent of this order).
		__global__ void __launch_bounds__(128) CellFlagsListedKernel(const float* __restrict__ lat, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, uint32_t* __restrict__ words,
			uint32_t* __restrict__ cells, uint32_t* __restrict__ cell_count)
		{
			const CellGeom cg = Geom(g);
			const uint32_t n = *count;
			const int lane = threadIdx.x & 31;
			for (uint32_t item = blockIdx.x; item < n; item += gridDim.x)
			{
				const BrickCells bc = CellsOf(__ldg(list + item), bg, cg);
				const int total = bc.nx * bc.ny * bc.nz;
				const int rounds = (total + (int)blockDim.x - 1) / (int)blockDim.x;
				for (int r = 0; r < rounds; ++r)
				{
					const int t = r * (int)blockDim.x + (int)threadIdx.x;
					bool active = false;
					int64_t c = 0;
					if (t < total)
					{
						const int64_t i = bc.i0 + t % bc.nx, j = bc.j0 + (t / bc.nx) % bc.ny, k = bc.k0 + t / (bc.nx * bc.ny);
						float v[8];
						LoadCorners(lat, cg, i, j, k, v);
						unsigned pos = 0;
#pragma unroll
						for (int q = 0; q < 8; ++q) pos |= (v[q] >= 0.0f ? 1u : 0u) << q;
						active = pos != 0u && pos != 0xFFu;
						c = i + j * cg.sx + k * cg.sx * cg.sy;
						if (active) atomicOr(words + (c >> 5), 1u << (c & 31));
					}
					const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
					uint32_t base = 0;
					if (lane == 0 && ballot) base = atomicAdd(cell_count, (uint32_t)__popc(ballot));
					base = __shfl_sync(0xFFFFFFFFu, base, 0);
					if (active) cells[base + __popc(ballot & ((1u << lane) - 1u))] = (uint32_t)c;
				}
			}
		}

		// One thread per active cell of the list: its vertex number is its rank in the
		// bitmask, so the output is in cell order whatever the list order.
		__global__ void __launch_bounds__(128) CellVerticesListedKernel(const float* __restrict__ lat, GridSpec g,
			const uint32_t* __restrict__ cells, uint32_t cell_count, const uint32_t* __restrict__ words,
			const uint32_t* __restrict__ base, float* __restrict__ vertices, uint32_t* __restrict__ cubes,
			uint32_t* __restrict__ face_counts)
		{
			const CellGeom cg = Geom(g);
			const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
			if (t >= cell_count) return;
			const int64_t c = __ldg(cells + t);
			const uint32_t w = __ldg(words + (c >> 5));
			const uint32_t vid = __ldg(base + (c >> 5)) + __popc(w & ((1u << (c & 31)) - 1u));
			const int64_t i = c % cg.sx, j = (c / cg.sx) % cg.sy, k = c / (cg.sx * cg.sy);
			EmitCellVertex(lat, g, cg, words, c, i, j, k, vid, vertices, cubes, face_counts);
		}

		BrickGrid MakeBrickGrid(const GridSpec& g, int B)
		{
			return { B, (g.NX - 1 + B - 1) / B, (g.NY - 1 + B - 1) / B, (g.NZ - 1 + B - 1) / B };
		}
	}

	int64_t BrickCount(const GridSpec& g, int B)
	{
		const BrickGrid bg = MakeBrickGrid(g, B);
		return (int64_t)bg.NBX * bg.NBY * bg.NBZ;
	}

	cudaError_t LaunchClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, uint32_t* brick_bits, uint32_t* list,
		uint32_t* count, cudaStream_t stream)
	{
		const BrickGrid bg = MakeBrickGrid(g, B);
		const int64_t nb = (int64_t)bg.NBX * bg.NBY * bg.NBZ;
		cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t), stream);
		if (e != cudaSuccess) return e;
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depth * kClassifyThreads * sizeof(float);
		if (smem > 48 * 1024) cudaFuncSetAttribute(ClassifyBricksKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		ClassifyBricksKernel<<<(unsigned)((nb + kClassifyThreads - 1) / kClassifyThreads), kClassifyThreads, smem, stream>>>(
			prog, g, bg, brick_bits, list, count);
		return cudaGetLastError();
	}

	namespace
	{
		template<int C, int K>
		cudaError_t LaunchEvalBricksCK(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
			float* lattice, int grid_blocks, cudaStream_t stream)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			const size_t smem = (size_t)depth * K * kBrickThreads * sizeof(float);
			if (smem > 48 * 1024)
			{
				cudaError_t e = cudaFuncSetAttribute(EvalBricksKernel<C, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
				if (e != cudaSuccess) return e;
			}
			EvalBricksKernel<C, K><<<grid_blocks, kBrickThreads, smem, stream>>>(prog, g, MakeBrickGrid(g, B), list, count, lattice);
			return cudaGetLastError();
		}

		template<int C>
		cudaError_t LaunchEvalBricksC(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
			float* lattice, int grid_blocks, cudaStream_t stream, int lanes)
		{
			switch (lanes)
			{
			case 1: return LaunchEvalBricksCK<C, 1>(prog, g, B, list, count, lattice, grid_blocks, stream);
			case 2: return LaunchEvalBricksCK<C, 2>(prog, g, B, list, count, lattice, grid_blocks, stream);
			default: return LaunchEvalBricksCK<C, 4>(prog, g, B, list, count, lattice, grid_blocks, stream);
			}
		}
	}

	cudaError_t LaunchEvalBricks(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		float* lattice, int grid_blocks, cudaStream_t stream, int lanes)
	{
		if (B + 1 <= 8) return LaunchEvalBricksC<8>(prog, g, B, list, count, lattice, grid_blocks, stream, lanes);
		if (B + 1 <= 16) return LaunchEvalBricksC<16>(prog, g, B, list, count, lattice, grid_blocks, stream, lanes);
		return cudaErrorInvalidValue;
	}

	cudaError_t LaunchCellFlagsBricks(const float* lattice, const GridSpec& g, int B, const uint32_t* brick_bits, uint32_t* words,
		cudaStream_t stream)
	{
		const BrickGrid bg = MakeBrickGrid(g, B);
		const int64_t cells = (int64_t)(g.NX - 1) * (g.NY - 1) * (g.NZ - 1);
		if (cells <= 0) return cudaSuccess;
		CellFlagsBricksKernel<<<(unsigned)((cells + 255) / 256), 256, 0, stream>>>(lattice, g, bg, brick_bits, words, cells);
		return cudaGetLastError();
	}

	cudaError_t LaunchCellFlagsListed(const float* lattice, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		uint32_t* words, uint32_t* cells, uint32_t* cell_count, int grid_blocks, cudaStream_t stream)
	{
		const int64_t total = (int64_t)(g.NX - 1) * (g.NY - 1) * (g.NZ - 1);
		cudaError_t e = cudaMemsetAsync(words, 0, (size_t)((total + 31) / 32) * 4, stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(cell_count, 0, sizeof(uint32_t), stream);
		if (e != cudaSuccess) return e;
		CellFlagsListedKernel<<<grid_blocks, 128, 0, stream>>>(lattice, g, MakeBrickGrid(g, B), list, count, words, cells, cell_count);
		return cudaGetLastError();
	}

	cudaError_t LaunchCellVerticesListed(const float* lattice, const GridSpec& g, const uint32_t* cells, uint32_t cell_count,
		const uint32_t* words, const uint32_t* word_base, float* vertices, uint32_t* cubes, uint32_t* face_counts, cudaStream_t stream)
	{
		if (cell_count == 0) return cudaSuccess;
		CellVerticesListedKernel<<<(cell_count + 127) / 128, 128, 0, stream>>>(lattice, g, cells, cell_count, words, word_base,
			vertices, cubes, face_counts);
		return cudaGetLastError();
	}
}
