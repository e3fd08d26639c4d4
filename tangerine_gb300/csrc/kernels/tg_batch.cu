// Many trees exported in one persistent launch.
//
// Every model's bricks, cells and vertices live in one global index space: model m owns
// brick-bit words [BrickWord0, BrickWord0 + BrickWords), cell-bit words from CellWord0,
// lattice floats from Lattice, and (after the cell scan) vertices from VertexBase[m].  A
// cooperative grid runs the export's phases over that space -- classify bricks, list the
// survivors, evaluate them, flag active cells, number the vertices, emit vertices, number
// and emit faces, gradient normals and colours -- separated by grid-wide barriers, so the
// work queue of (model, brick) items balances models of very different sizes across the
// whole GPU.  Per model, the results are exactly the single-model export's: the same
// kernels' per-item code, vertices in cell order, faces holding the model's own vertex
// numbers.
//
// The grid barrier is a counter and a generation word in global memory, waited on with a
// time limit: a barrier that runs out sets the status and every block leaves.  The last
// block to arrive at a barrier also reads the host's cancel flag; when it is set, every
// block leaves after that barrier.
#include <cstdint>

#include "tg_cull.cuh"
#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_surface.cuh"

namespace tg
{
	namespace
	{
		constexpr int kThreads = 128;
		constexpr int kScanItems = 4;
		constexpr uint64_t kBarrierLimitNs = 5000000000ull;    // 5 s

		__device__ __forceinline__ uint64_t Now()
		{
			uint64_t t;
			asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
			return t;
		}

		// Grid-wide barrier of a cooperative launch.  False (for every thread of the block)
		// when the wait ran out, the run was cancelled, or an earlier barrier failed.
		__device__ bool GridSync(const BatchState& s)
		{
			__shared__ int ok;
			__syncthreads();
			if (threadIdx.x == 0)
			{
				ok = 1;
				volatile unsigned* gen = s.Barrier + 1;
				const unsigned g = *gen;
				__threadfence();
				if (atomicAdd(s.Barrier, 1u) == gridDim.x - 1)
				{
					// Every block has arrived: the cancel decision is taken once, here, and
					// published with the status before the release.
					if (s.Cancel && *s.Cancel != 0) atomicCAS(s.Status, 0, 3);
					atomicExch(s.Barrier, 0u);
					__threadfence();
					atomicAdd(s.Barrier + 1, 1u);
				}
				else
				{
					const uint64_t limit = (s.Knobs && s.Knobs[0]) ? s.Knobs[0] : kBarrierLimitNs;
					const uint64_t t0 = Now();
					while (*gen == g)
					{
						if (*(volatile int*)s.Status != 0 || Now() - t0 > limit)
						{
							atomicCAS(s.Status, 0, 2);
							ok = 0;
							break;
						}
					}
				}
				__threadfence();
				if (*(volatile int*)s.Status != 0) ok = 0;
			}
			__syncthreads();
			return ok != 0;
		}

		// Index of the last model whose first item (starts[m]) is <= x.
		template<typename T>
		__device__ __forceinline__ int ModelOf(const T* __restrict__ starts, int count, T x)
		{
			int lo = 0, hi = count - 1;
			while (lo < hi)
			{
				const int mid = (lo + hi + 1) >> 1;
				if (__ldg(starts + mid) <= x) lo = mid;
				else hi = mid - 1;
			}
			return lo;
		}

		// ---- block and grid scans ------------------------------------------------------

		__device__ __forceinline__ uint32_t BlockScan(uint32_t x, uint32_t& total)
		{
			__shared__ uint32_t warpSums[kThreads / 32];
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
			uint32_t before = 0;
			total = 0;
#pragma unroll
			for (int w = 0; w < kThreads / 32; ++w)
			{
				const uint32_t v = warpSums[w];
				if (w < warp) before += v;
				total += v;
			}
			__syncthreads();
			return before + inc - x;
		}

		__device__ __forceinline__ uint32_t Item(const uint32_t* in, int64_t i, int64_t n, bool pop)
		{
			if (i >= n) return 0u;
			const uint32_t x = in[i];
			return pop ? (uint32_t)__popc(x) : x;
		}

		// Exclusive prefix sum over n items (popcounts of words, or values) into out; the
		// total lands in *total.  Three barriers.  `partials` holds gridDim.x + 1 words.
		__device__ bool GridScan(const BatchState& s, const uint32_t* in, int64_t n, bool pop, uint32_t* out, uint32_t* total)
		{
			const int64_t tile = (int64_t)kThreads * kScanItems;
			int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
			chunk = (chunk + tile - 1) / tile * tile;
			const int64_t b0 = (int64_t)blockIdx.x * chunk;
			const int64_t b1 = b0 + chunk < n ? b0 + chunk : n;
			{
				uint32_t sum = 0;
				for (int64_t i = b0 + threadIdx.x; i < b1; i += kThreads) sum += Item(in, i, n, pop);
				uint32_t t;
				BlockScan(sum, t);
				if (threadIdx.x == 0) s.ScanPartials[blockIdx.x] = t;
			}
			if (!GridSync(s)) return false;
			if (blockIdx.x == 0)
			{
				uint32_t carry = 0;
				for (int64_t base = 0; base < gridDim.x; base += kThreads)
				{
					const int64_t i = base + threadIdx.x;
					const uint32_t v = i < gridDim.x ? s.ScanPartials[i] : 0u;
					uint32_t t;
					const uint32_t ex = BlockScan(v, t);
					if (i < gridDim.x) s.ScanPartials[i] = carry + ex;
					carry += t;
				}
				if (threadIdx.x == 0)
				{
					s.ScanPartials[gridDim.x] = carry;
					*total = carry;
				}
			}
			if (!GridSync(s)) return false;
			uint32_t run = s.ScanPartials[blockIdx.x];
			for (int64_t base = b0; base < b1; base += tile)
			{
				uint32_t v[kScanItems];
				uint32_t local = 0;
				const int64_t first = base + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
				for (int q = 0; q < kScanItems; ++q)
				{
					v[q] = first + q < b1 ? Item(in, first + q, n, pop) : 0u;
					local += v[q];
				}
				uint32_t t;
				uint32_t ex = BlockScan(local, t) + run;
#pragma unroll
				for (int q = 0; q < kScanItems; ++q)
				{
					if (first + q < b1) out[first + q] = ex;
					ex += v[q];
				}
				run += t;
			}
			return GridSync(s);
		}

		// ---- per-item work ---------------------------------------------------------------

		template<int K>
		__device__ void EvalBrickK(const BatchModel& m, float* __restrict__ lattice, uint32_t b, uint32_t packed_top, float* spill)
		{
			// The brick's descent from phase 2: every point below the cell reached by the whole
			// box, and only where the box straddles a pivot a per-point descent from there.
			const int top = (int)(packed_top & 0x7FFFFFFFu);
			const bool shared = (packed_top >> 31) != 0u;
			const GridSpec& g = m.Grid;
			const DeviceProgram& prog = m.Prog;
			constexpr int ZSpan = 2 * K;
			const int tx = threadIdx.x & 7, ty = (threadIdx.x >> 3) & 7, tz = threadIdx.x >> 6;
			const int bx = (int)(b % (uint32_t)m.NBX), by = (int)((b / (uint32_t)m.NBX) % (uint32_t)m.NBY);
			const int bz = (int)(b / ((uint32_t)m.NBX * (uint32_t)m.NBY));
			const int i0 = bx * m.B, j0 = by * m.B, k0 = bz * m.B;
			const int i1 = min(i0 + m.B, g.NX - 1), j1 = min(j0 + m.B, g.NY - 1), k1 = min(k0 + m.B, g.NZ - 1);
			for (int oz = 0; oz <= k1 - k0; oz += ZSpan)
			for (int oy = 0; oy <= j1 - j0; oy += 8)
			for (int ox = 0; ox <= i1 - i0; ox += 8)
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
					RunDistance<K, false>(prog.Code, __ldg(&prog.Nodes[c].DistanceCode), px, py, pz, r, spill + threadIdx.x, kThreads);
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

		// ---- the persistent kernel ---------------------------------------------------------

		// Compiled for 8 resident CTAs per SM (64 registers): at the default 80 registers the
		// interpreter loops spilled about 1.2 KB a thread and the 512-tree batch took 140 ms;
		// at 64 it spills 0.16 KB, outside the record loops, and takes 124 ms.
		__global__ void __launch_bounds__(kThreads, 8) BatchExportKernel(BatchState s)
		{
			extern __shared__ float spill[];
			const int warpsPerGrid = gridDim.x * (kThreads / 32);
			const int warp = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
			const int lane = threadIdx.x & 31;
			const int64_t gthreads = (int64_t)gridDim.x * kThreads;
			const int64_t gtid = (int64_t)blockIdx.x * kThreads + threadIdx.x;

			// Test hook (tg_batch_debug_barrier): one block starts late, by at most 2 s, so the
			// other blocks' first barrier wait can be made to run out.
			if (s.Knobs && s.Knobs[1] == (uint64_t)blockIdx.x + 1 && threadIdx.x == 0)
			{
				const uint64_t delay = s.Knobs[2] < 2000000000ull ? s.Knobs[2] : 2000000000ull;
				const uint64_t t0 = Now();
				while (Now() - t0 < delay) __nanosleep(1000);
			}

			// 1. Classify every brick of every model; clear the cell bits.  Exact models go by
			//    8 x 4 patches of neighbouring bricks (a warp each, bits set with atomicOr into
			//    words zeroed first), which keeps a warp on one holder program.  Models culled
			//    by a learned bound arrive with their bits set by it (a warp per bit word):
			//    those keep them (Cull 1) or put the kept bricks through the exact test (Cull 2).
			for (int64_t w = gtid; w < s.BrickWordsTotal; w += gthreads)
			{
				if (s.Models[ModelOf(s.BrickWord0, s.Count, w)].Cull == 0) s.BrickBits[w] = 0u;
			}
			for (int64_t w = gtid; w < s.CellWordsTotal; w += gthreads) s.CellBits[w] = 0u;
			if (!GridSync(s)) return;
			for (int64_t t = warp; t < s.TilesTotal; t += warpsPerGrid)
			{
				const int mi = ModelOf(s.Tile0, s.Count, t);
				const BatchModel& m = s.Models[mi];
				if (m.Cull != 0) continue;
				const int64_t local = t - __ldg(s.Tile0 + mi);
				const int tilesX = (m.NBX + 7) / 8, tilesY = (m.NBY + 3) / 4;
				const int bx = (int)(local % tilesX) * 8 + (lane & 7);
				const int by = (int)((local / tilesX) % tilesY) * 4 + (lane >> 3);
				const int bz = (int)(local / ((int64_t)tilesX * tilesY));
				if (bx < m.NBX && by < m.NBY)
				{
					const int i0 = bx * m.B, j0 = by * m.B, k0 = bz * m.B;
					if (BoxMayHoldSurface<false>(m.Prog, m.Grid, i0, min(i0 + m.B, m.Grid.NX - 1), j0, min(j0 + m.B, m.Grid.NY - 1),
						k0, min(k0 + m.B, m.Grid.NZ - 1), spill + threadIdx.x, kThreads))
					{
						const int64_t b = bx + (int64_t)m.NBX * (by + (int64_t)m.NBY * bz);
						atomicOr(s.BrickBits + m.BrickWord0 + (b >> 5), 1u << (b & 31));
					}
				}
			}
			for (int64_t w = warp; w < s.BrickWordsTotal; w += warpsPerGrid)
			{
				const int mi = ModelOf(s.BrickWord0, s.Count, w);
				const BatchModel& m = s.Models[mi];
				if (m.Cull == 0) continue;
				const int64_t local = (w - m.BrickWord0) * 32 + lane;
				bool active = false;
				const bool candidate = ((s.BrickBits[w] >> lane) & 1u) != 0;
				if (local < m.Bricks && candidate && m.Cull == 1)
				{
					active = true;
				}
				else if (local < m.Bricks && candidate)
				{
					const int bx = (int)(local % m.NBX), by = (int)((local / m.NBX) % m.NBY), bz = (int)(local / ((int64_t)m.NBX * m.NBY));
					const int i0 = bx * m.B, j0 = by * m.B, k0 = bz * m.B;
					active = BoxMayHoldSurface<false>(m.Prog, m.Grid, i0, min(i0 + m.B, m.Grid.NX - 1), j0, min(j0 + m.B, m.Grid.NY - 1),
						k0, min(k0 + m.B, m.Grid.NZ - 1), spill + threadIdx.x, kThreads);
				}
				const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
				if (lane == 0) s.BrickBits[w] = ballot;
			}
			if (!GridSync(s)) return;

			// 2. Kept bricks as a list, the costliest programs first (cost classes of the
			//    bricks' descended cells, as the single export's list): bricks with long
			//    programs drawn last would leave the end of phase 3 to a few CTAs.  A thread
			//    per brick-bit word, its kept bricks one per round; counts per class with one
			//    atomic per class and warp, then the places.
			uint32_t* classCounts = s.Counters + 8;
			uint32_t* classCursors = s.Counters + 12;
			for (int64_t w = gtid; w - (int64_t)lane < s.BrickWordsTotal; w += gthreads)
			{
				uint32_t bits = w < s.BrickWordsTotal ? s.BrickBits[w] : 0u;
				const BatchModel* m = bits ? &s.Models[ModelOf(s.BrickWord0, s.Count, w)] : nullptr;
				while (__any_sync(0xFFFFFFFFu, bits != 0u))
				{
					int cls = kCostClasses;
					if (bits)
					{
						const int j = __ffs((int)bits) - 1;
						bits &= bits - 1u;
						const int64_t gb = w * 32 + j;
						const int64_t b = gb - m->BrickWord0 * 32;
						const int bx = (int)(b % m->NBX), by = (int)((b / m->NBX) % m->NBY), bz = (int)(b / ((int64_t)m->NBX * m->NBY));
						const int i0 = bx * m->B, j0 = by * m->B, k0 = bz * m->B;
						const uint32_t top = BrickTop(m->Prog, m->Grid, i0, min(i0 + m->B, m->Grid.NX - 1), j0, min(j0 + m->B, m->Grid.NY - 1),
							k0, min(k0 + m->B, m->Grid.NZ - 1));
						s.BrickTops[gb] = top;
						cls = CostClass(m->Prog, top);
					}
					const unsigned peers = __match_any_sync(0xFFFFFFFFu, cls);
					if (cls < kCostClasses && lane == __ffs((int)peers) - 1)
					{
						atomicAdd(classCounts + cls, (uint32_t)__popc(peers));
						atomicAdd(s.Counters + 0, (uint32_t)__popc(peers));
					}
				}
			}
			if (!GridSync(s)) return;
			uint32_t classStart[kCostClasses];
			{
				uint32_t o = 0;
#pragma unroll
				for (int c = 0; c < kCostClasses; ++c) { classStart[c] = o; o += classCounts[c]; }
			}
			for (int64_t w = gtid; w - (int64_t)lane < s.BrickWordsTotal; w += gthreads)
			{
				uint32_t bits = w < s.BrickWordsTotal ? s.BrickBits[w] : 0u;
				const BatchModel* m = bits ? &s.Models[ModelOf(s.BrickWord0, s.Count, w)] : nullptr;
				while (__any_sync(0xFFFFFFFFu, bits != 0u))
				{
					int cls = kCostClasses;
					int64_t gb = 0;
					if (bits)
					{
						const int j = __ffs((int)bits) - 1;
						bits &= bits - 1u;
						gb = w * 32 + j;
						cls = CostClass(m->Prog, s.BrickTops[gb]);
					}
					const unsigned peers = __match_any_sync(0xFFFFFFFFu, cls);
					if (cls < kCostClasses)
					{
						const int leader = __ffs((int)peers) - 1;
						uint32_t at = 0;
						if (lane == leader) at = atomicAdd(classCursors + cls, (uint32_t)__popc(peers));
						at = __shfl_sync(peers, at, leader);
						uint32_t start = classStart[0];
#pragma unroll
						for (int c = 1; c < kCostClasses; ++c) if (cls == c) start = classStart[c];
						s.BrickList[start + at + (uint32_t)__popc(peers & ((1u << lane) - 1u))] = (uint32_t)gb;
					}
				}
			}
			if (!GridSync(s)) return;
			const uint32_t kept = s.Counters[0];

			// 3. Distances at the lattice points of every kept brick (a CTA per brick).
			for (uint32_t item = blockIdx.x; item < kept; item += gridDim.x)
			{
				const uint32_t gb = s.BrickList[item];
				const int mi = ModelOf(s.BrickWord0, s.Count, (int64_t)(gb >> 5));
				const BatchModel& m = s.Models[mi];
				const uint32_t b = gb - (uint32_t)(m.BrickWord0 * 32);
				float* lat = s.Lattice + m.Lattice;
				const uint32_t top = s.BrickTops[gb];
				if (m.Lanes == 1) EvalBrickK<1>(m, lat, b, top, spill);
				else if (m.Lanes == 4) EvalBrickK<4>(m, lat, b, top, spill);
				else EvalBrickK<2>(m, lat, b, top, spill);
			}
			if (!GridSync(s)) return;

			// 4. Active cells of the kept bricks: bits, and an append list of global cell bits.
			//    Bricks of at most 7^3 cells (every brick size the tuner picks) stage their
			//    lattice box in shared memory and append their cells with one atomic.
			{
				__shared__ float box[8 * 8 * 8];
				__shared__ uint32_t warpBase[kThreads / 32];
				for (uint32_t item = blockIdx.x; item < kept; item += gridDim.x)
				{
					const uint32_t gb = s.BrickList[item];
					const int mi = ModelOf(s.BrickWord0, s.Count, (int64_t)(gb >> 5));
					const BatchModel& m = s.Models[mi];
					const uint32_t b = gb - (uint32_t)(m.BrickWord0 * 32);
					const CellGeom cg = Geom(m.Grid);
					const float* lat = s.Lattice + m.Lattice;
					const int bx = (int)(b % (uint32_t)m.NBX), by = (int)((b / (uint32_t)m.NBX) % (uint32_t)m.NBY);
					const int bz = (int)(b / ((uint32_t)m.NBX * (uint32_t)m.NBY));
					const int64_t ci0 = (int64_t)bx * m.B, cj0 = (int64_t)by * m.B, ck0 = (int64_t)bz * m.B;
					const int nx = (int)min((int64_t)m.B, cg.sx - ci0), ny = (int)min((int64_t)m.B, cg.sy - cj0);
					const int nz = (int)min((int64_t)m.B, cg.sz - ck0);
					const int total = nx * ny * nz;
					if (m.B <= 7)
					{
						__syncthreads();   // the previous brick is done with the box and the bases
						for (int t = (int)threadIdx.x; t < 512; t += kThreads)
						{
							const int x = t & 7, y = (t >> 3) & 7, z = t >> 6;
							if (x <= nx && y <= ny && z <= nz) box[t] = __ldg(lat + ((ck0 + z) * cg.ny + cj0 + y) * cg.nx + ci0 + x);
						}
						__syncthreads();
						constexpr int kRounds = 3;   // 7^3 = 343 cells <= 3 x 128
						unsigned ballots[kRounds];
						uint64_t cellOf[kRounds];
						uint32_t count = 0;
#pragma unroll
						for (int r = 0; r < kRounds; ++r)
						{
							const int t = r * kThreads + (int)threadIdx.x;
							bool active = false;
							cellOf[r] = 0;
							if (t < total)
							{
								const int x = t % nx, y = (t / nx) % ny, z = t / (nx * ny);
								const float* q = box + (z * 8 + y) * 8 + x;
								const float v[8] = { q[0], q[1], q[9], q[8], q[64], q[65], q[73], q[72] };
								unsigned pos = 0;
#pragma unroll
								for (int k = 0; k < 8; ++k) pos |= (v[k] >= 0.0f ? 1u : 0u) << k;
								active = pos != 0u && pos != 0xFFu;
								const int64_t c = (ci0 + x) + (cj0 + y) * cg.sx + (ck0 + z) * cg.sx * cg.sy;
								if (active) atomicOr(s.CellBits + m.CellWord0 + (c >> 5), 1u << (c & 31));
								cellOf[r] = (uint64_t)m.CellWord0 * 32u + (uint64_t)c;
							}
							ballots[r] = __ballot_sync(0xFFFFFFFFu, active);
							count += (uint32_t)__popc(ballots[r]);
						}
						if (lane == 0) warpBase[threadIdx.x >> 5] = count;
						__syncthreads();
						if (threadIdx.x == 0)
						{
							uint32_t counts[kThreads / 32], sum = 0;
#pragma unroll
							for (int w = 0; w < kThreads / 32; ++w) { counts[w] = warpBase[w]; sum += counts[w]; }
							uint32_t at = sum ? atomicAdd(s.Counters + 1, sum) : 0u;
#pragma unroll
							for (int w = 0; w < kThreads / 32; ++w) { warpBase[w] = at; at += counts[w]; }
						}
						__syncthreads();
						uint32_t at = warpBase[threadIdx.x >> 5];
						const unsigned below = (1u << lane) - 1u;
#pragma unroll
						for (int r = 0; r < kRounds; ++r)
						{
							const uint32_t slot = at + (uint32_t)__popc(ballots[r] & below);
							if (((ballots[r] >> lane) & 1u) && slot < s.CapVertices) s.ActiveCells[slot] = cellOf[r];
							at += (uint32_t)__popc(ballots[r]);
						}
						continue;
					}
					for (int r0 = 0; r0 < total; r0 += kThreads)
					{
						const int t = r0 + (int)threadIdx.x;
						bool active = false;
						int64_t c = 0;
						if (t < total)
						{
							const int64_t i = ci0 + t % nx, j = cj0 + (t / nx) % ny, k = ck0 + t / (nx * ny);
							float v[8];
							LoadCorners(lat, cg, i, j, k, v);
							unsigned pos = 0;
#pragma unroll
							for (int q = 0; q < 8; ++q) pos |= (v[q] >= 0.0f ? 1u : 0u) << q;
							active = pos != 0u && pos != 0xFFu;
							c = i + j * cg.sx + k * cg.sx * cg.sy;
							if (active) atomicOr(s.CellBits + m.CellWord0 + (c >> 5), 1u << (c & 31));
						}
						const unsigned ballot = __ballot_sync(0xFFFFFFFFu, active);
						uint32_t base = 0;
						if (lane == 0 && ballot) base = atomicAdd(s.Counters + 1, (uint32_t)__popc(ballot));
						base = __shfl_sync(0xFFFFFFFFu, base, 0);
						const uint32_t at = base + __popc(ballot & ((1u << lane) - 1u));
						if (active && at < s.CapVertices) s.ActiveCells[at] = (uint64_t)m.CellWord0 * 32u + (uint64_t)c;
					}
				}
			}
			if (!GridSync(s)) return;

			// 5. Vertex numbers: ranks in the global cell bitmask.
			if (!GridScan(s, s.CellBits, s.CellWordsTotal, true, s.CellWordBase, s.Counters + 2)) return;
			const uint32_t vertices = s.Counters[2];
			const bool vertexRoom = vertices <= s.CapVertices;
			if (!vertexRoom && gtid == 0) atomicOr(s.Counters + 4, 1u);

			// 6. Vertices, cube numbers and face counts; each model's first vertex.
			for (int64_t mi = gtid; mi <= s.Count; mi += gthreads)
			{
				if (mi == s.Count) s.VertexBase[mi] = vertices;
				else s.VertexBase[mi] = s.CellWords[mi] ? s.CellWordBase[s.Models[mi].CellWord0] : vertices;
			}
			if (vertexRoom)
			{
				const uint32_t active = s.Counters[1] < s.CapVertices ? s.Counters[1] : s.CapVertices;
				for (int64_t t = gtid; t < active; t += gthreads)
				{
					const uint64_t gc = s.ActiveCells[t];
					const int m2 = ModelOf(s.CellBit0, s.Count, gc);
					const BatchModel& m = s.Models[m2];
					const int64_t c = (int64_t)(gc - (uint64_t)m.CellWord0 * 32u);
					const CellGeom cg = Geom(m.Grid);
					const uint32_t* words = s.CellBits + m.CellWord0;
					const uint32_t* base = s.CellWordBase + m.CellWord0;
					const uint32_t w = words[c >> 5];
					const uint32_t vid = base[c >> 5] + __popc(w & ((1u << (c & 31)) - 1u));
					const int64_t i = c % cg.sx, j = (c / cg.sx) % cg.sy, k = c / (cg.sx * cg.sy);
					EmitCellVertex(s.Lattice + m.Lattice, m.Grid, cg, words, c, i, j, k, vid, s.Vertices, s.Cubes, s.FaceCounts);
				}
			}
			if (!GridSync(s)) return;

			// 7. Face numbers.
			if (!GridScan(s, s.FaceCounts, vertexRoom ? vertices : 0, false, s.FaceBase, s.Counters + 3)) return;
			const uint32_t faces = s.Counters[3];
			const bool faceRoom = vertexRoom && faces <= s.CapFaces;
			if (!faceRoom && gtid == 0) atomicOr(s.Counters + 4, 2u);
			for (int64_t mi = gtid; mi <= s.Count; mi += gthreads)
			{
				const uint32_t v = s.VertexBase[mi];
				s.FaceBaseModel[mi] = (mi == s.Count || v >= vertices || !vertexRoom) ? faces : s.FaceBase[v];
			}

			// 8. Triangles, numbered within their model.
			if (faceRoom)
			{
				for (int64_t v0 = gtid; v0 < vertices; v0 += gthreads)
				{
					const int mi = ModelOf(s.VertexBase, s.Count, (uint32_t)v0);
					const BatchModel& m = s.Models[mi];
					const CellGeom cg = Geom(m.Grid);
					const float* lat = s.Lattice + m.Lattice;
					const uint32_t* words = s.CellBits + m.CellWord0;
					const uint32_t* base = s.CellWordBase + m.CellWord0;
					const uint32_t vb = s.VertexBase[mi];
					const int64_t c = s.Cubes[v0];
					const int64_t i = c % cg.sx, j = (c / cg.sx) % cg.sy, k = c / (cg.sx * cg.sy);
					if (i == 0 || j == 0 || k == 0) continue;
					const int64_t dy = cg.sx, dz = cg.sx * cg.sy;
					const int64_t nb[6] = { c - 1, c - 1 - dy, c - dy, c - dy - dz, c - dz, c - 1 - dz };
					const int quads[3][3] = { {0, 1, 2}, {0, 5, 4}, {2, 3, 4} };
					const float c0 = Corner(lat, cg, i, j, k);
					const float sv[3][2] = { { c0, Corner(lat, cg, i, j, k + 1) }, { Corner(lat, cg, i, j + 1, k), c0 },
						{ c0, Corner(lat, cg, i + 1, j, k) } };
					uint32_t out = s.FaceBase[v0];
					const uint32_t self = (uint32_t)v0 - vb;
					for (int q = 0; q < 3; ++q)
					{
						const int64_t a = nb[quads[q][0]], b = nb[quads[q][1]], d = nb[quads[q][2]];
						if (!(IsActive(words, a) && IsActive(words, b) && IsActive(words, d))) continue;
						const uint32_t nv[3] = { VertexOf(words, base, a) - vb, VertexOf(words, base, b) - vb, VertexOf(words, base, d) - vb };
						uint32_t v1, v2, v3;
						if (sv[q][1] > sv[q][0]) { v1 = nv[0]; v2 = nv[1]; v3 = nv[2]; }
						else { v1 = nv[2]; v2 = nv[1]; v3 = nv[0]; }
						uint32_t* f = s.Faces + (int64_t)out * 3;
						f[0] = self; f[1] = v1; f[2] = v2;
						f[3] = self; f[4] = v2; f[5] = v3;
						out += 2;
					}
				}
			}

			// 9. Gradient normals (four lanes per vertex, one tetrahedral offset each, all
			//    running the same code; the vertex itself only when the four cancel), then
			//    colours (one thread per vertex of a painted model, GetMaterial's walk).
			if (s.Attributes && vertexRoom)
			{
				constexpr int kNormalPoints = kThreads / 4;
				const int localPoint = threadIdx.x >> 2, elane = threadIdx.x & 3;
				const int groupFirst = (lane & ~3);
				for (int64_t first = (int64_t)blockIdx.x * kNormalPoints; first < vertices; first += (int64_t)gridDim.x * kNormalPoints)
				{
					const int64_t v = first + localPoint;
					const bool mine = v < vertices;
					float e = 0.0f;
					int mi = 0, pc = 0;
					Vec3 p(0.0f, 0.0f, 0.0f);
					if (mine)
					{
						mi = ModelOf(s.VertexBase, s.Count, (uint32_t)v);
						const BatchModel& m = s.Models[mi];
						p = Vec3(s.Vertices[v * 3], s.Vertices[v * 3 + 1], s.Vertices[v * 3 + 2]);
						const int cell = DescendOctree(m.Prog.Nodes, p.x, p.y, p.z);
						pc = __ldg(&m.Prog.Nodes[cell].SurfaceCode);
						const Vec3 q = TetraPoint(p, elane);
						const float px[1] = { q.x }, py[1] = { q.y }, pz[1] = { q.z };
						float r[1];
						RunSurfaceBatch<1, false>(m.Prog.Code, pc, px, py, pz, r, -1, nullptr, spill + threadIdx.x, kThreads);
						e = r[0];
					}
					float ev[5];
#pragma unroll
					for (int j = 0; j < 4; ++j) ev[j] = __shfl_sync(0xFFFFFFFFu, e, groupFirst + j);
					if (mine && elane == 0)
					{
						const BatchModel& m = s.Models[mi];
						ev[4] = 0.0f;
						const float h = 0.0001f;
						const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
						Vec3 g = xyy * ev[0];
						g = g + yyx * ev[1];
						g = g + yxy * ev[2];
						g = g + xxx * ev[3];
						if ((g.x * g.x + g.y * g.y) + g.z * g.z == 0.0f)
						{
							const float qx[1] = { p.x }, qy[1] = { p.y }, qz[1] = { p.z };
							float r[1];
							RunSurfaceBatch<1, false>(m.Prog.Code, pc, qx, qy, qz, r, -1, nullptr, spill + threadIdx.x, kThreads);
							ev[4] = r[0];
						}
						const Vec3 n = GradientOf(ev);
						s.Normals[v * 3 + 0] = n.x;
						s.Normals[v * 3 + 1] = n.y;
						s.Normals[v * 3 + 2] = n.z;
					}
				}
				for (int64_t v = gtid; v < vertices; v += gthreads)
				{
					const int mi = ModelOf(s.VertexBase, s.Count, (uint32_t)v);
					const BatchModel& m = s.Models[mi];
					if (!m.HasPaint) continue;
					const Vec3 p(s.Vertices[v * 3], s.Vertices[v * 3 + 1], s.Vertices[v * 3 + 2]);
					const int cell = DescendOctree(m.Prog.Nodes, p.x, p.y, p.z);
					const int pc = __ldg(&m.Prog.Nodes[cell].SurfaceCode);
					const float px[1] = { p.x }, py[1] = { p.y }, pz[1] = { p.z };
					float r[1];
					int mt = -1;
					RunSurfaceBatch<1, false>(m.Prog.Code, pc, px, py, pz, r, 0, &mt, spill + threadIdx.x, kThreads);
					const uchar4 c = mt >= 0 ? m.Prog.Colors[mt] : make_uchar4(255, 255, 255, 255);
					s.Colors[v * 3 + 0] = c.x;
					s.Colors[v * 3 + 1] = c.y;
					s.Colors[v * 3 + 2] = c.z;
				}
			}
		}
	}

	size_t BatchSharedBytes(int max_stack)
	{
		const int depth = max_stack > 1 ? max_stack - 1 : 1;
		return (size_t)depth * 4 * kThreads * sizeof(float);      // K = 4 lanes of distance spill
	}

	int BatchThreads() { return kThreads; }

	cudaError_t BatchMaxBlocks(int max_stack, int* blocks)
	{
		const size_t smem = BatchSharedBytes(max_stack);
		cudaError_t e = cudaFuncSetAttribute(BatchExportKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		int perSm = 0, dev = 0, sms = 0;
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, BatchExportKernel, kThreads, smem);
		if (e == cudaSuccess) e = cudaGetDevice(&dev);
		if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (e != cudaSuccess) return e;
		*blocks = perSm * sms;
		return cudaSuccess;
	}

	cudaError_t LaunchBatchExport(const BatchState& s, int blocks, int max_stack, cudaStream_t stream)
	{
		const size_t smem = BatchSharedBytes(max_stack);
		cudaError_t e = cudaFuncSetAttribute(BatchExportKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		BatchState copy = s;
		void* args[] = { &copy };
		return cudaLaunchCooperativeKernel((const void*)BatchExportKernel, dim3(blocks), dim3(kThreads), args, smem, stream);
	}
}
