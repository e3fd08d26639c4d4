// Per-cell pieces of naive surface nets shared by the dense and the brick-culled passes
// (third_party/naive-surface-nets/src/surface_nets.cpp:864-1121).
#pragma once

#include "tg_device.cuh"

namespace tg
{
	struct CellGeom
	{
		int64_t sx, sy, sz;     // cells per axis
		int64_t nx, ny;         // lattice points per axis (x, y)
	};

	__device__ __forceinline__ CellGeom Geom(const GridSpec& g)
	{
		return { g.NX - 1, g.NY - 1, g.NZ - 1, g.NX, g.NY };
	}

	__device__ __forceinline__ float Corner(const float* __restrict__ lat, const CellGeom& cg, int64_t i, int64_t j, int64_t k)
	{
		return __ldg(lat + (k * cg.ny + j) * cg.nx + i);
	}

	// Corner order and edge list of the reference (surface_nets.cpp:889-901).
	static __constant__ int8_t kCornerOfs[8][3] = { {0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1} };
	static __constant__ int8_t kEdges[12][2] = { {0,1},{1,2},{2,3},{3,0},{4,5},{5,6},{6,7},{7,4},{0,4},{1,5},{2,6},{3,7} };

	__device__ __forceinline__ void LoadCorners(const float* __restrict__ lat, const CellGeom& cg, int64_t i, int64_t j, int64_t k, float (&v)[8])
	{
		const int64_t base = (k * cg.ny + j) * cg.nx + i;
		const int64_t dy = cg.nx, dz = cg.nx * cg.ny;
		v[0] = __ldg(lat + base);
		v[1] = __ldg(lat + base + 1);
		v[2] = __ldg(lat + base + dy + 1);
		v[3] = __ldg(lat + base + dy);
		v[4] = __ldg(lat + base + dz);
		v[5] = __ldg(lat + base + dz + 1);
		v[6] = __ldg(lat + base + dz + dy + 1);
		v[7] = __ldg(lat + base + dz + dy);
	}

	__device__ __forceinline__ bool IsActive(const uint32_t* __restrict__ words, int64_t cell)
	{
		return (__ldg(words + (cell >> 5)) >> (cell & 31)) & 1u;
	}

	__device__ __forceinline__ uint32_t VertexOf(const uint32_t* __restrict__ words, const uint32_t* __restrict__ base, int64_t cell)
	{
		const uint32_t w = __ldg(words + (cell >> 5));
		return __ldg(base + (cell >> 5)) + __popc(w & ((1u << (cell & 31)) - 1u));
	}


	// FirstLoopInnerThunk's vertex (surface_nets.cpp:915-965) for active cell c = (i, j, k)
	// at its rank `vid`, and the number of triangles SecondLoopThunk will emit for it
	// (surface_nets.cpp:1016-1115).
	__device__ __forceinline__ void EmitCellVertex(const float* __restrict__ lat, const GridSpec& g, const CellGeom& cg,
		const uint32_t* __restrict__ words, int64_t c, int64_t i, int64_t j, int64_t k, uint32_t vid,
		float* __restrict__ vertices, uint32_t* __restrict__ cubes, uint32_t* __restrict__ face_counts)
	{
		float v[8];
		LoadCorners(lat, cg, i, j, k, v);
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
		const float fsx = (float)cg.sx, fsy = (float)cg.sy, fsz = (float)cg.sz;
		const float maxx = g.X0 + fsx * g.DX, maxy = g.Y0 + fsy * g.DY, maxz = g.Z0 + fsz * g.DZ;
		vertices[(int64_t)vid * 3 + 0] = g.X0 + (maxx - g.X0) * (cx - 0.0f) / (fsx - 0.0f);
		vertices[(int64_t)vid * 3 + 1] = g.Y0 + (maxy - g.Y0) * (cy - 0.0f) / (fsy - 0.0f);
		vertices[(int64_t)vid * 3 + 2] = g.Z0 + (maxz - g.Z0) * (cz - 0.0f) / (fsz - 0.0f);
		cubes[vid] = (uint32_t)c;

		uint32_t faces = 0;
		if (i > 0 && j > 0 && k > 0)
		{
			const int64_t dy = cg.sx, dz = cg.sx * cg.sy;
			// neighbours 0..5: (i-1,j,k) (i-1,j-1,k) (i,j-1,k) (i,j-1,k-1) (i,j,k-1) (i-1,j,k-1)
			const bool n0 = IsActive(words, c - 1), n1 = IsActive(words, c - 1 - dy), n2 = IsActive(words, c - dy);
			const bool n3 = IsActive(words, c - dy - dz), n4 = IsActive(words, c - dz), n5 = IsActive(words, c - 1 - dz);
			if (n0 && n1 && n2) faces += 2;
			if (n0 && n5 && n4) faces += 2;
			if (n2 && n3 && n4) faces += 2;
		}
		face_counts[vid] = faces;
	}

	// SDFNode::Gradient's evaluation points (sdf_evaluator.cpp:298-333): the four
	// tetrahedral offsets for lanes 0..3, the point itself for lane 4.
	__device__ __forceinline__ Vec3 TetraPoint(Vec3 p, int lane)
	{
		const float h = 0.0001f;
		switch (lane)
		{
		case 0: return p + Vec3(h, -h, -h);
		case 1: return p + Vec3(-h, -h, h);
		case 2: return p + Vec3(-h, h, -h);
		case 3: return p + Vec3(h, h, h);
		default: return p;
		}
	}

	// SDFNode::Gradient (sdf_evaluator.cpp:298-333) from the five evaluations.
	__device__ __forceinline__ Vec3 GradientOf(const float* e)
	{
		const float h = 0.0001f;
		const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
		Vec3 g = xyy * e[0];
		g = g + yyx * e[1];
		g = g + yxy * e[2];
		g = g + xxx * e[3];
		const float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
		if (ls == 0.0f)
		{
			const float d = e[4];
			return Normalize(Vec3(e[0] - d, e[2] - d, e[1] - d));
		}
		return g / sqrtf(ls);
	}
}
