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
#include "tg_cull.cuh"
#include "tg_pair.cuh"
#include "tg_tc.cuh"

namespace tg
{
	namespace
	{
		constexpr int kClassifyThreads = 128;
		constexpr int kBrickThreads = 128;     // 8 x 8 columns x 2 z-groups of 4 points
		// Resident CTAs per SM the brick evaluation is compiled for (48 registers a thread).
		// 7^3-cell bricks, 512^3 export: 0.65 ms at 8 (64 registers), 0.58 at 9, 0.56 at 10,
		// 0.66 at 12 (spills).  32^3-cell bricks, 1024^3 export: 56.1 -> 63.3 G samples/s
		// (network-culled) from 8 to 10.
		template<int C> constexpr int EvalBricksCtasPerSm() { return 10; }
		constexpr int kCellPassCtasPerSm = 16;
		constexpr int kListedCtasPerSm = 8;

		struct BrickGrid
		{
			int B;                  // cells per brick edge
			int NBX, NBY, NBZ;      // bricks per axis
		};

		// A CTA takes a tile of 8 x 4 x 4 bricks and each warp an 8 x 4 patch of it: the
		// bricks of a warp are neighbours in space, so they mostly run the same holder
		// program (a warp along a row of 32 bricks spans several octree cells and diverges).
		// Kept bricks set their bit with atomicOr into the zeroed bit words.
		constexpr int kTileX = 8, kTileY = 4, kTileZ = kClassifyThreads / (kTileX * kTileY);

		__global__ void __launch_bounds__(kClassifyThreads) ClassifyBricksKernel(DeviceProgram prog, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ candidates, uint32_t* __restrict__ brick_bits, uint32_t* __restrict__ brick_tops)
		{
			extern __shared__ float spill[];
			const int tilesX = (bg.NBX + kTileX - 1) / kTileX, tilesY = (bg.NBY + kTileY - 1) / kTileY;
			const int tile = (int)blockIdx.x;
			const int bx = (tile % tilesX) * kTileX + (int)(threadIdx.x % kTileX);
			const int by = ((tile / tilesX) % tilesY) * kTileY + (int)((threadIdx.x / kTileX) % kTileY);
			const int bz = (tile / (tilesX * tilesY)) * kTileZ + (int)(threadIdx.x / (kTileX * kTileY));
			if (bx >= bg.NBX || by >= bg.NBY || bz >= bg.NBZ) return;
			const int64_t b = bx + (int64_t)bg.NBX * (by + (int64_t)bg.NBY * bz);
			if (candidates && !((__ldg(candidates + (b >> 5)) >> (b & 31)) & 1u)) return;
			const int sx = g.NX - 1, sy = g.NY - 1, sz = g.NZ - 1;
			const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
			const int i1 = min(i0 + bg.B, sx), j1 = min(j0 + bg.B, sy), k1 = min(k0 + bg.B, sz);
			if (BoxMayHoldSurface(prog, g, i0, i1, j0, j1, k0, k1, spill + threadIdx.x, kClassifyThreads))
			{
				atomicOr(brick_bits + (b >> 5), 1u << (b & 31));
				if (brick_tops) brick_tops[b] = BrickTop(prog, g, i0, i1, j0, j1, k0, k1);
			}
		}

		// Kept bricks by cost class, a thread per brick.  Place = false adds each class's
		// bricks to counts[c] and all of them to *total; Place = true (counts[0..3] complete,
		// counts[4..7] zeroed) writes class c's bricks after those of the classes before it,
		// in about brick-index order within a class (warps append in the order they run).
		// Descend (with Place = false): the kept bricks' descents are not stored yet; each
		// thread writes its brick's into tops first, for the placing pass and the evaluation.
		template<bool Place, bool Descend>
		__global__ void ListBricksByCostKernel(const uint32_t* __restrict__ bits, int64_t bricks, DeviceProgram prog, GridSpec g,
			BrickGrid bg, uint32_t* __restrict__ tops, uint32_t* counts, uint32_t* total, uint32_t* __restrict__ list)
		{
			const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			const int lane = (int)(threadIdx.x & 31);
			int cls = kCostClasses;           // not kept
			if (b < bricks && ((__ldg(bits + (b >> 5)) >> (b & 31)) & 1u))
			{
				uint32_t top;
				if constexpr (Descend)
				{
					const int bx = (int)(b % bg.NBX), by = (int)((b / bg.NBX) % bg.NBY), bz = (int)(b / ((int64_t)bg.NBX * bg.NBY));
					const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
					top = BrickTop(prog, g, i0, min(i0 + bg.B, g.NX - 1), j0, min(j0 + bg.B, g.NY - 1), k0, min(k0 + bg.B, g.NZ - 1));
					tops[b] = top;
				}
				else
				{
					top = __ldg(tops + b);
				}
				cls = CostClass(prog, top);
			}
			const unsigned peers = __match_any_sync(0xFFFFFFFFu, cls);
			if (cls == kCostClasses) return;
			const int leader = __ffs((int)peers) - 1;
			const uint32_t k = (uint32_t)__popc(peers);
			if (!Place)
			{
				if (lane == leader) { atomicAdd(counts + cls, k); atomicAdd(total, k); }
				return;
			}
			uint32_t at = 0;
			if (lane == leader) at = atomicAdd(counts + kCostClasses + cls, k);
			at = __shfl_sync(peers, at, leader);
			uint32_t start = 0;
#pragma unroll
			for (int c = 0; c < kCostClasses - 1; ++c) if (c < cls) start += counts[c];
			list[start + at + (uint32_t)__popc(peers & ((1u << lane) - 1u))] = (uint32_t)b;
		}

		// Bricks whose bit is set, in brick-index order (x fastest): consecutive list entries
		// are neighbours, so the CTAs evaluating them at the same time share octree cells and
		// their record streams in cache.
		__global__ void ListBricksKernel(const uint32_t* __restrict__ bits, int64_t words, const uint32_t* __restrict__ base,
			uint32_t* __restrict__ list)
		{
			const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (w >= words) return;
			uint32_t m = bits[w];
			uint32_t at = base[w];
			while (m)
			{
				const int j = __ffs(m) - 1;
				m &= m - 1u;
				list[at++] = (uint32_t)(w * 32 + j);
			}
		}

		constexpr int kBrickWarps = kBrickThreads / 32;

		// Test hook of the staged-copy wait (SetStageWaitTest): nonzero, a staging warp first
		// waits this long on an mbarrier that nothing arrives at, so the wait runs out as a
		// copy that never completes would.
		__device__ unsigned long long g_stage_wait_test_ns = 0;

		// One slice of a brick (see EvalBricksKernel): lane `lane` runs its column's K
		// z-consecutive points of every 8 x 8 x 2K block of the brick's box, through one pass
		// over their octree cell's records per distinct cell.  `code`: the records (read with
		// __ldg, or with generic loads when Generic: a staged copy).  Box: the values also go
		// to `box`, the brick's C^3 corner box in shared memory (x fastest), for the cell pass
		// folded into EvalBricksCellsKernel.
		template<int C, int K, bool Generic, bool Box>
		__device__ __forceinline__ void EvalSlice(const DeviceProgram& prog, const GridSpec& g, int i0, int i1, int j0, int j1, int k0,
			int k1, int top, bool shared, int slice, int lane, const float4* code, float* __restrict__ lattice, float* spill, float* box)
		{
			constexpr int ZSpan = 2 * K;
			const int tx = lane & 7, ty = (lane >> 3) + 4 * (slice & 1), tz = slice >> 1;
			for (int oz = 0; oz < C; oz += ZSpan)
			for (int oy = 0; oy < C; oy += 8)
			for (int ox = 0; ox < C; ox += 8)
			{
				const int ix = i0 + ox + tx, iy = j0 + oy + ty, izb = k0 + oz + tz * K;
				const bool inPlane = ix <= i1 && iy <= j1;
				const float x = LatticeCoord(g.X0, min(ix, i1), g.DX);
				const float y = LatticeCoord(g.Y0, min(iy, j1), g.DY);
				float px[K], py[K], pz[K], res[K];
				int cell[K];
				unsigned todo = 0;
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					const int iz = izb + k;
					px[k] = x;
					py[k] = y;
					pz[k] = LatticeCoord(g.Z0, min(iz, k1), g.DZ);
					cell[k] = shared ? top : DescendOctreeFrom(prog.Nodes, top, px[k], py[k], pz[k]);
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
					if constexpr (K % 2 == 0)
					{
						// Points in pairs through the paired FP32 instructions (tg_pair.cuh).
						if (Generic)
						{
							RunDistancePaired<K>([&](int q) { return code[q]; }, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r,
								spill + 2 * threadIdx.x, kBrickThreads);
						}
						else
						{
							RunDistancePaired<K>([&](int q) { return __ldg(code + q); }, __ldg(&prog.Nodes[c].DistanceCode), px,
								py, pz, r, spill + 2 * threadIdx.x, kBrickThreads);
						}
					}
					else
					{
						RunDistance<K>(prog.Code, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r, spill + threadIdx.x, kBrickThreads);
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
						const int iz = izb + k;
						if (iz <= k1)
						{
							lattice[((int64_t)iz * g.NY + iy) * g.NX + ix] = res[k];
							if (Box) box[((oz + tz * K + k) * C + (oy + ty)) * C + (ox + tx)] = res[k];
						}
					}
				}
			}
		}

		// Lattice points of every listed brick: corners [i0, i0 + B] per axis, clamped to the
		// lattice.  A brick's box is covered in 8 x 8 column blocks x 2 z-groups: a brick has
		// four slices, slice s holding rows 4 (s & 1) .. 4 (s & 1) + 3 of each 8 x 8 block and
		// z-group s >> 1; a lane runs K z-consecutive points of its column through one pass
		// over their octree cell's records, so one pass of a slice covers an 8 x 4 x K box.
		// A warp draws (brick, slice) items from a counter and goes on to its next item when it
		// is done; a brick's cost follows its cell programs' lengths, and the list holds the
		// costliest bricks first (LaunchListBricks), so the launch does not end on them.  The
		// four slices of a brick are consecutive items, so they mostly run at the same time
		// and share the records in L1.
		// Stage = true: a warp whose brick's points all descend to one octree cell (the common
		// case) first copies that cell's distance program into its own shared memory with one
		// bulk copy (cp.async.bulk, completion on the warp's mbarrier, bounded wait) and reads
		// the records there; other bricks read them from global memory.  Both go through one
		// generic-address load, so the interpreter is compiled once.
		template<int C, int K, bool Stage>
		__global__ void __launch_bounds__(kBrickThreads, EvalBricksCtasPerSm<C>()) EvalBricksKernel(DeviceProgram prog, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, const uint32_t* __restrict__ tops,
			float* __restrict__ lattice, int spill_floats, int stage_quads, int* __restrict__ status, uint32_t* __restrict__ next)
		{
			extern __shared__ __align__(16) float spill[];
			__shared__ uint64_t staged_bar[kBrickWarps], idle_bar[kBrickWarps];
			const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
			float4* staged = reinterpret_cast<float4*>(spill + spill_floats) + warp * stage_quads;
			uint32_t phase = 0;
			if (Stage && lane == 0)
			{
				tc::BarInit(&staged_bar[warp], 1);
				tc::BarInit(&idle_bar[warp], 1);
			}
			__syncwarp();
			// Items: a lattice that fits the device has fewer than 2^30 bricks.
			const uint32_t items = *count * (uint32_t)kBrickWarps;
			for (;;)
			{
				uint32_t item = 0;
				if (lane == 0) item = atomicAdd(next, 1u);
				item = __shfl_sync(0xffffffffu, item, 0);
				if (item >= items) break;
				const int slice = (int)(item % kBrickWarps);
				const uint32_t b = __ldg(list + item / kBrickWarps);
				const int bx = (int)(b % (uint32_t)bg.NBX), by = (int)((b / (uint32_t)bg.NBX) % (uint32_t)bg.NBY);
				const int bz = (int)(b / ((uint32_t)bg.NBX * (uint32_t)bg.NBY));
				const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
				const int i1 = min(i0 + bg.B, g.NX - 1), j1 = min(j0 + bg.B, g.NY - 1), k1 = min(k0 + bg.B, g.NZ - 1);
				// The brick's points mostly share one octree cell: the descent with the brick's
				// box (lattice coordinates are monotone in the index; the classifier's, when it
				// stored one), then per point only below where the box straddles a pivot.
				const uint32_t packed = tops ? __ldg(tops + b) : BrickTop(prog, g, i0, i1, j0, j1, k0, k1);
				const int top = (int)(packed & 0x7FFFFFFFu);
				const bool shared = (packed >> 31) != 0u;
				// Record reads go through `code` (generic address): the staged copy, offset so that
				// the program's own record numbers index it, or the program's global records.
				const float4* code = prog.Code;
				if (Stage && shared)
				{
					const int dc = __ldg(&prog.Nodes[top].DistanceCode);
					const int len = __ldg(&prog.Nodes[top].SurfaceCode) - dc;
					if (len > 0 && len <= stage_quads)
					{
						if (lane == 0) tc::BulkLoad(staged, prog.Code + dc, (uint32_t)len * 16u, &staged_bar[warp]);
						const uint64_t testLimit = g_stage_wait_test_ns;
						const bool ok = testLimit ? tc::BarWaitFor(&idle_bar[warp], 0, testLimit) : tc::BarWait(&staged_bar[warp], phase);
						if (!ok)
						{
							// The copy did not complete in time: report it, wait (bounded) for the
							// copy still in flight, and leave.
							atomicExch(status, 1);
							tc::BarWait(&staged_bar[warp], phase);
							return;
						}
						phase ^= 1u;
						code = staged - dc;
					}
				}
				EvalSlice<C, K, Stage, false>(prog, g, i0, i1, j0, j1, k0, k1, top, shared, slice, lane, code, lattice, spill, nullptr);
				__syncwarp();   // every lane is done with this item's staged copy
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

		// The same pass for bricks of at most 7^3 cells: the CTA first stages the brick's
		// lattice box (at most 8^3 points, coalesced rows) in shared memory, so each cell
		// reads its eight corners there instead of issuing eight scattered global loads, and
		// the brick's active cells take their slots in `cells` with one atomic per brick.
		constexpr int kTiledBox = 8;
		constexpr int kTiledThreads = 128;
		constexpr int kTiledRounds = 3;   // 7^3 = 343 cells <= 3 x 128

		// BT: the brick edge in cells when known at compile time (the cell coordinates then
		// come from constant divisions, edge bricks masking their missing cells), or 0.
		// The cell pass of one kept brick from its corner box in shared memory (kTiledBox^3,
		// x fastest): every cell with corners of both signs sets its bit in `words` and is
		// appended to `cells` (one atomic per brick).  Called by the whole CTA (it
		// synchronises); `warpBase` is shared scratch, one word per warp.
		template<int BT>
		__device__ __forceinline__ void BrickCellFlags(const float* box, const BrickCells& bc, const CellGeom& cg, uint32_t* __restrict__ words,
			uint32_t* __restrict__ cells, uint32_t* __restrict__ cell_count, uint32_t* warpBase)
		{
			const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
			const int ex = BT ? BT : bc.nx, ey = BT ? BT : bc.ny;
			const int total = BT ? BT * BT * BT : bc.nx * bc.ny * bc.nz;
			const int64_t sxy = cg.sx * cg.sy;
			const int64_t c0 = bc.i0 + bc.j0 * cg.sx + bc.k0 * sxy;
			unsigned ballots[kTiledRounds];
			uint32_t cellOf[kTiledRounds];
			uint32_t mine = 0;
#pragma unroll
			for (int r = 0; r < kTiledRounds; ++r)
			{
				const int t = r * kTiledThreads + (int)threadIdx.x;
				bool active = false;
				cellOf[r] = 0;
				const int x = t % ex, y = (t / ex) % ey, z = t / (ex * ey);
				if (t < total && x < bc.nx && y < bc.ny && z < bc.nz)
				{
					const float* b = box + (z * kTiledBox + y) * kTiledBox + x;
					constexpr int dy = kTiledBox, dz = kTiledBox * kTiledBox;
					const float v[8] = { b[0], b[1], b[dy + 1], b[dy], b[dz], b[dz + 1], b[dz + dy + 1], b[dz + dy] };
					unsigned pos = 0;
#pragma unroll
					for (int q = 0; q < 8; ++q) pos |= (v[q] >= 0.0f ? 1u : 0u) << q;
					active = pos != 0u && pos != 0xFFu;
					const int64_t c = c0 + x + y * cg.sx + z * sxy;
					cellOf[r] = (uint32_t)c;
					if (active) atomicOr(words + (c >> 5), 1u << (c & 31));
				}
				ballots[r] = __ballot_sync(0xFFFFFFFFu, active);
				mine += (uint32_t)__popc(ballots[r]);
			}
			if (lane == 0) warpBase[warp] = mine;
			__syncthreads();
			if (threadIdx.x == 0)
			{
				uint32_t sum = 0;
				uint32_t counts[kTiledThreads / 32];
#pragma unroll
				for (int w = 0; w < kTiledThreads / 32; ++w) { counts[w] = warpBase[w]; sum += counts[w]; }
				uint32_t at = sum ? atomicAdd(cell_count, sum) : 0u;
#pragma unroll
				for (int w = 0; w < kTiledThreads / 32; ++w) { warpBase[w] = at; at += counts[w]; }
			}
			__syncthreads();
			uint32_t at = warpBase[warp];
			const unsigned below = (1u << lane) - 1u;
#pragma unroll
			for (int r = 0; r < kTiledRounds; ++r)
			{
				if ((ballots[r] >> lane) & 1u) cells[at + __popc(ballots[r] & below)] = cellOf[r];
				at += (uint32_t)__popc(ballots[r]);
			}
		}

		template<int BT>
		__global__ void __launch_bounds__(kTiledThreads) CellFlagsTiledKernel(const float* __restrict__ lat, GridSpec g, BrickGrid bg,
			const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, uint32_t* __restrict__ words,
			uint32_t* __restrict__ cells, uint32_t* __restrict__ cell_count)
		{
			__shared__ float box[kTiledBox * kTiledBox * kTiledBox];
			__shared__ uint32_t warpBase[kTiledThreads / 32];
			const CellGeom cg = Geom(g);
			const uint32_t n = *count;
			for (uint32_t item = blockIdx.x; item < n; item += gridDim.x)
			{
				const BrickCells bc = CellsOf(__ldg(list + item), bg, cg);
				__syncthreads();   // the previous brick is done with the box and the bases
				for (int t = (int)threadIdx.x; t < kTiledBox * kTiledBox * kTiledBox; t += kTiledThreads)
				{
					const int x = t & 7, y = (t >> 3) & 7, z = t >> 6;
					if (x <= bc.nx && y <= bc.ny && z <= bc.nz)
						box[t] = __ldg(lat + ((bc.k0 + z) * cg.ny + bc.j0 + y) * cg.nx + bc.i0 + x);
				}
				__syncthreads();
				BrickCellFlags<BT>(box, bc, cg, words, cells, cell_count, warpBase);
			}
		}

		// The brick evaluation with the cell pass folded in (7^3-cell bricks, programs read
		// from global memory): a CTA draws a brick from a counter, each warp evaluates one of
		// its four slices (EvalSlice) into the lattice and into the brick's 8^3 corner box in
		// shared memory, and the CTA then flags and lists the brick's active cells from that
		// box (BrickCellFlags) -- the separate cell pass read the boxes back from memory.
		template<int K>
		__global__ void __launch_bounds__(kBrickThreads, EvalBricksCtasPerSm<8>()) EvalBricksCellsKernel(DeviceProgram prog, GridSpec g,
			BrickGrid bg, const uint32_t* __restrict__ list, const uint32_t* __restrict__ count, const uint32_t* __restrict__ tops,
			float* __restrict__ lattice, uint32_t* __restrict__ words, uint32_t* __restrict__ cells, uint32_t* __restrict__ cell_count,
			uint32_t* __restrict__ next)
		{
			extern __shared__ __align__(16) float spill[];
			__shared__ float box[kTiledBox * kTiledBox * kTiledBox];
			__shared__ uint32_t warpBase[kBrickWarps];
			__shared__ uint32_t itemSlot;
			static_assert(kBrickWarps == kTiledThreads / 32, "the cell pass takes the CTA's warps");
			const CellGeom cg = Geom(g);
			const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
			const uint32_t n = *count;
			for (;;)
			{
				if (threadIdx.x == 0) itemSlot = atomicAdd(next, 1u);
				__syncthreads();   // also: the previous brick is done with the box and the bases
				const uint32_t item = itemSlot;
				__syncthreads();
				if (item >= n) break;
				const uint32_t b = __ldg(list + item);
				const int bx = (int)(b % (uint32_t)bg.NBX), by = (int)((b / (uint32_t)bg.NBX) % (uint32_t)bg.NBY);
				const int bz = (int)(b / ((uint32_t)bg.NBX * (uint32_t)bg.NBY));
				const int i0 = bx * bg.B, j0 = by * bg.B, k0 = bz * bg.B;
				const int i1 = min(i0 + bg.B, g.NX - 1), j1 = min(j0 + bg.B, g.NY - 1), k1 = min(k0 + bg.B, g.NZ - 1);
				const uint32_t packed = tops ? __ldg(tops + b) : BrickTop(prog, g, i0, i1, j0, j1, k0, k1);
				EvalSlice<8, K, false, true>(prog, g, i0, i1, j0, j1, k0, k1, (int)(packed & 0x7FFFFFFFu), (packed >> 31) != 0u, warp, lane,
					prog.Code, lattice, spill, box);
				__syncthreads();
				BrickCellFlags<kTiledBox - 1>(box, CellsOf(b, bg, cg), cg, words, cells, cell_count, warpBase);
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

	cudaError_t LaunchClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, uint32_t* brick_bits, cudaStream_t stream,
		const uint32_t* candidates, uint32_t* brick_tops)
	{
		const BrickGrid bg = MakeBrickGrid(g, B);
		const int64_t nb = (int64_t)bg.NBX * bg.NBY * bg.NBZ;
		if (nb <= 0) return cudaSuccess;
		const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
		const size_t smem = (size_t)depth * kClassifyThreads * sizeof(float);
		if (smem > 48 * 1024) cudaFuncSetAttribute(ClassifyBricksKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		cudaError_t e = cudaMemsetAsync(brick_bits, 0, (size_t)((nb + 31) / 32) * 4, stream);
		if (e != cudaSuccess) return e;
		const int64_t tiles = (int64_t)((bg.NBX + kTileX - 1) / kTileX) * ((bg.NBY + kTileY - 1) / kTileY) * ((bg.NBZ + kTileZ - 1) / kTileZ);
		ClassifyBricksKernel<<<(unsigned)tiles, kClassifyThreads, smem, stream>>>(prog, g, bg, candidates, brick_bits, brick_tops);
		return cudaGetLastError();
	}

	cudaError_t LaunchListBricks(const uint32_t* brick_bits, int64_t bricks, uint32_t* base, uint32_t* scratch, uint32_t* list,
		uint32_t* count, cudaStream_t stream, const DeviceProgram* prog, uint32_t* tops, uint32_t* class_counts, const GridSpec* descend,
		int B)
	{
		const int64_t words = (bricks + 31) / 32;
		if (words <= 0) return cudaMemsetAsync(count, 0, 4, stream);
		if (prog && tops && class_counts)
		{
			GridSpec g{};
			BrickGrid bg{};
			if (descend)
			{
				g = *descend;
				bg = MakeBrickGrid(g, B);
				if ((int64_t)bg.NBX * bg.NBY * bg.NBZ != bricks) return cudaErrorInvalidValue;
			}
			cudaError_t e = cudaMemsetAsync(class_counts, 0, 2 * kCostClasses * sizeof(uint32_t), stream);
			if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(uint32_t), stream);
			if (e != cudaSuccess) return e;
			const unsigned blocks = (unsigned)((bricks + 255) / 256);
			if (descend)
				ListBricksByCostKernel<false, true><<<blocks, 256, 0, stream>>>(brick_bits, bricks, *prog, g, bg, tops, class_counts, count, list);
			else
				ListBricksByCostKernel<false, false><<<blocks, 256, 0, stream>>>(brick_bits, bricks, *prog, g, bg, tops, class_counts, count, list);
			ListBricksByCostKernel<true, false><<<blocks, 256, 0, stream>>>(brick_bits, bricks, *prog, g, bg, tops, class_counts, count, list);
			return cudaGetLastError();
		}
		cudaError_t e = LaunchExclusiveScan(brick_bits, words, true, base, count, scratch, stream);
		if (e != cudaSuccess) return e;
		ListBricksKernel<<<(unsigned)((words + 255) / 256), 256, 0, stream>>>(brick_bits, words, base, list);
		return cudaGetLastError();
	}

	namespace
	{
		// Shared memory of a CTA at the compiled occupancy, with a little left for the
		// runtime's reserve; the warps' staged programs get what the spill leaves.
		constexpr size_t kStageBudget = 20 * 1024;

		template<int C, int K, bool Stage>
		cudaError_t LaunchEvalBricksCKS(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
			const uint32_t* tops, float* lattice, int sms, cudaStream_t stream, int* status)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			const size_t spill = (size_t)depth * K * kBrickThreads * sizeof(float);
			int stageQuads = 0;
			if (Stage && spill + kBrickWarps * 16 * 16 <= kStageBudget) stageQuads = (int)((kStageBudget - spill) / (16 * kBrickWarps));
			const size_t smem = spill + (size_t)kBrickWarps * stageQuads * 16;
			if (smem > 48 * 1024)
			{
				cudaError_t e = cudaFuncSetAttribute(EvalBricksKernel<C, K, Stage>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
				if (e != cudaSuccess) return e;
			}
			EvalBricksKernel<C, K, Stage><<<sms * EvalBricksCtasPerSm<C>(), kBrickThreads, smem, stream>>>(prog, g, MakeBrickGrid(g, B), list,
				count, tops, lattice, (int)(spill / sizeof(float)), stageQuads, status, reinterpret_cast<uint32_t*>(status) + 1);
			return cudaGetLastError();
		}

		template<int C, int K>
		cudaError_t LaunchEvalBricksCK(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
			const uint32_t* tops, float* lattice, int sms, cudaStream_t stream, bool staged, int* status)
		{
			if (staged) return LaunchEvalBricksCKS<C, K, true>(prog, g, B, list, count, tops, lattice, sms, stream, status);
			return LaunchEvalBricksCKS<C, K, false>(prog, g, B, list, count, tops, lattice, sms, stream, status);
		}

		template<int C>
		cudaError_t LaunchEvalBricksC(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
			const uint32_t* tops, float* lattice, int sms, cudaStream_t stream, int lanes, bool staged, int* status)
		{
			switch (lanes)
			{
			case 1: return LaunchEvalBricksCK<C, 1>(prog, g, B, list, count, tops, lattice, sms, stream, staged, status);
			case 2: return LaunchEvalBricksCK<C, 2>(prog, g, B, list, count, tops, lattice, sms, stream, staged, status);
			default: return LaunchEvalBricksCK<C, 4>(prog, g, B, list, count, tops, lattice, sms, stream, staged, status);
			}
		}
	}

	cudaError_t SetStageWaitTest(uint64_t limit_ns)
	{
		const unsigned long long v = limit_ns;
		return cudaMemcpyToSymbol(g_stage_wait_test_ns, &v, sizeof(v));
	}

	cudaError_t LaunchEvalBricks(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		const uint32_t* tops, float* lattice, int sms, cudaStream_t stream, int lanes, bool staged, int* status)
	{
		if (B + 1 <= 8) return LaunchEvalBricksC<8>(prog, g, B, list, count, tops, lattice, sms, stream, lanes, staged, status);
		if (B + 1 <= 16) return LaunchEvalBricksC<16>(prog, g, B, list, count, tops, lattice, sms, stream, lanes, staged, status);
		if (B + 1 <= 24) return LaunchEvalBricksC<24>(prog, g, B, list, count, tops, lattice, sms, stream, lanes, staged, status);
		if (B + 1 <= 40) return LaunchEvalBricksC<40>(prog, g, B, list, count, tops, lattice, sms, stream, lanes, staged, status);
		return cudaErrorInvalidValue;
	}

	namespace
	{
		template<int K>
		cudaError_t LaunchEvalBricksCellsK(const DeviceProgram& prog, const GridSpec& g, const uint32_t* list, const uint32_t* count,
			const uint32_t* tops, float* lattice, uint32_t* words, uint32_t* cells, uint32_t* cell_count, int sms, cudaStream_t stream,
			int* status)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			const size_t smem = (size_t)depth * K * kBrickThreads * sizeof(float);
			if (smem > 40 * 1024)
			{
				cudaError_t e = cudaFuncSetAttribute(EvalBricksCellsKernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
				if (e != cudaSuccess) return e;
			}
			EvalBricksCellsKernel<K><<<sms * EvalBricksCtasPerSm<8>(), kBrickThreads, smem, stream>>>(prog, g, MakeBrickGrid(g, kTiledBox - 1),
				list, count, tops, lattice, words, cells, cell_count, reinterpret_cast<uint32_t*>(status) + 1);
			return cudaGetLastError();
		}
	}

	cudaError_t LaunchEvalBricksCells(const DeviceProgram& prog, const GridSpec& g, const uint32_t* list, const uint32_t* count,
		const uint32_t* tops, float* lattice, uint32_t* words, uint32_t* cells, uint32_t* cell_count, int sms, cudaStream_t stream,
		int lanes, int* status)
	{
		const int64_t total = (int64_t)(g.NX - 1) * (g.NY - 1) * (g.NZ - 1);
		cudaError_t e = cudaMemsetAsync(words, 0, (size_t)((total + 31) / 32) * 4, stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(cell_count, 0, sizeof(uint32_t), stream);
		if (e != cudaSuccess) return e;
		switch (lanes)
		{
		case 1: return LaunchEvalBricksCellsK<1>(prog, g, list, count, tops, lattice, words, cells, cell_count, sms, stream, status);
		case 2: return LaunchEvalBricksCellsK<2>(prog, g, list, count, tops, lattice, words, cells, cell_count, sms, stream, status);
		default: return LaunchEvalBricksCellsK<4>(prog, g, list, count, tops, lattice, words, cells, cell_count, sms, stream, status);
		}
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
		uint32_t* words, uint32_t* cells, uint32_t* cell_count, int sms, cudaStream_t stream)
	{
		const int64_t total = (int64_t)(g.NX - 1) * (g.NY - 1) * (g.NZ - 1);
		cudaError_t e = cudaMemsetAsync(words, 0, (size_t)((total + 31) / 32) * 4, stream);
		if (e == cudaSuccess) e = cudaMemsetAsync(cell_count, 0, sizeof(uint32_t), stream);
		if (e != cudaSuccess) return e;
		if (B == kTiledBox - 1)
			CellFlagsTiledKernel<kTiledBox - 1><<<sms * kCellPassCtasPerSm, kTiledThreads, 0, stream>>>(lattice, g, MakeBrickGrid(g, B), list,
				count, words, cells, cell_count);
		else if (B + 1 <= kTiledBox)
			CellFlagsTiledKernel<0><<<sms * kCellPassCtasPerSm, kTiledThreads, 0, stream>>>(lattice, g, MakeBrickGrid(g, B), list, count,
				words, cells, cell_count);
		else
			CellFlagsListedKernel<<<sms * kListedCtasPerSm, 128, 0, stream>>>(lattice, g, MakeBrickGrid(g, B), list, count, words, cells, cell_count);
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
