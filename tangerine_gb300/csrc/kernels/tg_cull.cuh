// Exact test of whether a lattice box may hold a sign change of the export distances
// (shared by the exact brick classifier and the network-assisted one).
#pragma once

#include "tg_device.cuh"
#include "tg_kernels.hpp"

namespace tg
{
	// Whether the lattice box [i0, i1] x [j0, j1] x [k0, k1] (corner indices) may hold a
	// sign change of the reference's distances; false only when that is proven.
	template<bool FuseSet = true>
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
		RunDistance<1, FuseSet>(prog.Code, __ldg(&prog.Nodes[holder].DistanceCode), px, py, pz, f, spill, stride);
		return !(fabsf(f[0]) > r + margin);
	}
}
