// Exact test of whether a lattice box may hold a sign change of the export distances
// (shared by the exact brick classifier and the network-assisted one).
#pragma once

#include "tg_device.cuh"
#include "tg_kernels.hpp"

namespace tg
{
	// The ball the exact test works with: the lattice box's bounding ball and the margin
	// that covers the rounding of its centre and of the programs.
	struct BoxBall
	{
		float cx, cy, cz, r, margin;
	};

	__device__ __forceinline__ BoxBall BallOfBox(const DeviceProgram& prog, const GridSpec& g, int i0, int i1, int j0, int j1, int k0, int k1)
	{
		const float x0 = LatticeCoord(g.X0, i0, g.DX), x1 = LatticeCoord(g.X0, i1, g.DX);
		const float y0 = LatticeCoord(g.Y0, j0, g.DY), y1 = LatticeCoord(g.Y0, j1, g.DY);
		const float z0 = LatticeCoord(g.Z0, k0, g.DZ), z1 = LatticeCoord(g.Z0, k1, g.DZ);
		BoxBall b;
		b.cx = 0.5f * (x0 + x1); b.cy = 0.5f * (y0 + y1); b.cz = 0.5f * (z0 + z1);
		const float ex = 0.5f * (x1 - x0), ey = 0.5f * (y1 - y0), ez = 0.5f * (z1 - z0);
		// Ball through the box's corners, widened for the rounding of the centre.
		b.r = sqrtf(ex * ex + ey * ey + ez * ez) * 1.0001f + 1e-6f;
		const float rootClip = __ldg(&prog.Nodes[0].ClipRadius);
		b.margin = 1e-4f * (1.0f + fabsf(b.cx) + fabsf(b.cy) + fabsf(b.cz) + fabsf(rootClip));
		return b;
	}

	constexpr int kBoxEmpty = -2;       // proven to hold no surface without a program
	constexpr int kBoxUndecided = -1;   // may hold surface: no cell's program can decide

	// The part of the exact test that needs no program: the root cube and dropped-octant
	// tests, then the deepest cell on the centre's descent path whose clip sphere holds
	// the ball (with no cell at or below it that is not 1-Lipschitz).  Returns that cell,
	// kBoxEmpty or kBoxUndecided.
	__device__ __forceinline__ int BoxHolder(const DeviceProgram& prog, const BoxBall& b)
	{
		const float rootClip = __ldg(&prog.Nodes[0].ClipRadius);
		// Outside the root cube every brush, and so every clipped program, is positive
		// (the cube holds the tree's bounds): a ball missing the cube has no surface.
		const float half = fabsf(rootClip) * 0.57736f;           // span / 2 = radius / sqrt(3), rounded up
		const float ox = fmaxf(fabsf(b.cx - __ldg(&prog.Nodes[0].Pivot[0])) - half, 0.0f);
		const float oy = fmaxf(fabsf(b.cy - __ldg(&prog.Nodes[0].Pivot[1])) - half, 0.0f);
		const float oz = fmaxf(fabsf(b.cz - __ldg(&prog.Nodes[0].Pivot[2])) - half, 0.0f);
		if (sqrtf(ox * ox + oy * oy + oz * oz) > b.r + b.margin) return kBoxEmpty;
		// Walking down, the holder is the deepest cell so far that holds the ball; a cell
		// that is not 1-Lipschitz voids the holders above it.
		int holder = kBoxUndecided;
		int at = 0;
		for (int guard = 0; guard < 48; ++guard)
		{
			const OctNode* n = prog.Nodes + at;
			const int32_t flags = __ldg(&n->Flags);
			const float px = __ldg(&n->Pivot[0]), py = __ldg(&n->Pivot[1]), pz = __ldg(&n->Pivot[2]);
			const float clip = __ldg(&n->ClipRadius);
			if (clip < 0.0f) holder = kBoxUndecided;
			else
			{
				const float dx = b.cx - px, dy = b.cy - py, dz = b.cz - pz;
				if (sqrtf(dx * dx + dy * dy + dz * dz) + b.r + b.margin <= clip) holder = at;
			}
			if (flags & kNodeTerminus) break;
			const int octant = (b.cx > px ? 1 : 0) | (b.cy > py ? 2 : 0) | (b.cz > pz ? 4 : 0);
			const int child = __ldg(&n->Child[octant]);
			if (child < 0)
			{
				// The octree dropped this octant because its clip returned null: the parent's
				// program exceeds the octant sphere's radius at its centre, so (1-Lipschitz) it
				// stays above the margin inside that sphere shrunk by the margin.  The octant
				// sphere sits inside the parent's, where the parent's program has the tree's
				// sign.  (Octants dropped because all their own children clipped away prove
				// only their cube, without margin, and are not used.)
				if (clip > 0.0f && ((flags >> (8 + octant)) & 1))
				{
					const float q = clip * 0.28867513f;               // span / 4 = radius / (2 sqrt 3)
					const float qx = px + ((octant & 1) ? q : -q), qy = py + ((octant & 2) ? q : -q), qz = pz + ((octant & 4) ? q : -q);
					const float dx = b.cx - qx, dy = b.cy - qy, dz = b.cz - qz;
					if (sqrtf(dx * dx + dy * dy + dz * dz) + b.r + b.margin <= clip * 0.4999f) return kBoxEmpty;
				}
				break;
			}
			at = child;
		}
		return holder;
	}

	// The holder cell's program at the ball's centre decides: |f| > r + margin proves no
	// sign change inside the ball.
	template<bool FuseSet = true>
	__device__ __forceinline__ bool HolderMayHoldSurface(const DeviceProgram& prog, int holder, const BoxBall& b, float* spill, int stride)
	{
		const float px[1] = { b.cx }, py[1] = { b.cy }, pz[1] = { b.cz };
		float f[1];
		RunDistance<1, FuseSet>(prog.Code, __ldg(&prog.Nodes[holder].DistanceCode), px, py, pz, f, spill, stride);
		return !(fabsf(f[0]) > b.r + b.margin);
	}

	// A kept brick's descent for the evaluation (DescendBox over its corner box): the cell
	// reached in the low 31 bits, bit 31 set when every point of the box descends to it.
	__device__ __forceinline__ uint32_t BrickTop(const DeviceProgram& prog, const GridSpec& g, int i0, int i1, int j0, int j1, int k0,
		int k1)
	{
		bool shared;
		const int top = DescendBox(prog.Nodes, LatticeCoord(g.X0, i0, g.DX), LatticeCoord(g.X0, i1, g.DX),
			LatticeCoord(g.Y0, j0, g.DY), LatticeCoord(g.Y0, j1, g.DY), LatticeCoord(g.Z0, k0, g.DZ),
			LatticeCoord(g.Z0, k1, g.DZ), shared);
		return (uint32_t)top | (shared ? 0x80000000u : 0u);
	}

	// Cost class of a kept brick, for the order the evaluation takes bricks in: the length
	// of its descended cell's distance program (for a brick whose box straddles a pivot,
	// an ancestor's, which is longer) in four classes, the longest first.  Bricks that
	// come last in brick-index order can be the costliest (long programs where the tree
	// is dense); taken last, one of them keeps its CTA busy long after the others are
	// done.
	constexpr int kCostClasses = 4;

	__device__ __forceinline__ int CostClass(const DeviceProgram& prog, uint32_t packed_top)
	{
		const int cell = (int)(packed_top & 0x7FFFFFFFu);
		const int len = __ldg(&prog.Nodes[cell].SurfaceCode) - __ldg(&prog.Nodes[cell].DistanceCode);
		return len >= 512 ? 0 : len >= 128 ? 1 : len >= 32 ? 2 : 3;
	}

	// Whether the lattice box [i0, i1] x [j0, j1] x [k0, k1] (corner indices) may hold a
	// sign change of the reference's distances; false only when that is proven.
	template<bool FuseSet = true>
	__device__ __forceinline__ bool BoxMayHoldSurface(const DeviceProgram& prog, const GridSpec& g,
		int i0, int i1, int j0, int j1, int k0, int k1, float* spill, int stride)
	{
		const BoxBall b = BallOfBox(prog, g, i0, i1, j0, j1, k0, k1);
		const int holder = BoxHolder(prog, b);
		if (holder == kBoxEmpty) return false;
		if (holder == kBoxUndecided) return true;
		return HolderMayHoldSurface<FuseSet>(prog, holder, b, spill, stride);
	}
}
