// Host side of Sodapop's meshing job (MeshingJob::NaiveSurfaceNets,
// tangerine/sodapop.cpp:562-897): the lattice and point-cache planning, and the kernel
// sequence of kernels/tg_sodapop.cu.
#include "tg_engine.hpp"

#include <cmath>

#define TG_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return _e; } while (0)

namespace tg
{
	namespace
	{
		// The reference's float loops over the aligned box count by ++ from an integer
		// value, which stays exact below 2^24.
		constexpr float kBoxLimit = 16777216.0f;

		bool AxisSpan(float lo, float hi, float origin, float step, int64_t& a, int64_t& b)
		{
			// glm::floor(glm::max(vec3(0), Min - Origin) / Step), glm::ceil((Max - Origin) / Step)
			const float amin = floorf(TernaryMax(0.0f, lo - origin) / step);
			const float amax = ceilf((hi - origin) / step);
			if (!(amin >= 0.0f && amin < kBoxLimit && amax > -kBoxLimit && amax < kBoxLimit)) return false;
			a = (int64_t)amin;
			b = (int64_t)amax;
			return true;
		}
	}

	bool SodapopPlan(const CompiledTree& t, float density, SodapopGrid& g, std::vector<int64_t>& boxes, std::string& error)
	{
		if (!std::isfinite(density))
		{
			error = "meshing density must be finite";
			return false;
		}
		// NaiveSurfaceNetsScratch (sodapop.cpp:153-177) on the octree root's bounds.
		const AABB& B = t.OctreeBounds;
		const Vec3 ext = B.Max - B.Min;
		const float fl = floorf(density);
		const Vec3 spu = TernaryMax(ext * Vec3(fl), Vec3(8.0f));
		const float cx = ceilf(spu.x), cy = ceilf(spu.y), cz = ceilf(spu.z);
		if (!(cx < 1.0e6f && cy < 1.0e6f && cz < 1.0e6f))
		{
			error = "meshing lattice too large";
			return false;
		}
		int64_t sx = (int64_t)cx, sy = (int64_t)cy, sz = (int64_t)cz;
		const float dx = ext.x / (float)sx, dy = ext.y / (float)sy, dz = ext.z / (float)sz;
		g.G[0] = B.Min.x - dx * 2.0f;
		g.G[1] = B.Min.y - dy * 2.0f;
		g.G[2] = B.Min.z - dz * 2.0f;
		g.D[0] = dx; g.D[1] = dy; g.D[2] = dz;
		sx += 3; sy += 3; sz += 3;
		g.SX = sx; g.SY = sy; g.SZ = sz;
		// The point cache's buckets (sodapop.cpp:613-620): 64 numbers each (fewer for a
		// tiny lattice); a number is kept when its bucket exists.
		const int64_t range = sx * sy * sz;
		const int64_t bucket = range < 64 ? range : 64;
		g.Limit = (range + bucket - 1) / bucket * bucket;
		if (g.Limit >= ((int64_t)1 << 31))
		{
			error = "meshing lattice has more cells than 32-bit vertex cell numbers hold";
			return false;
		}
		g.LZ = (g.Limit - 1) / (sx * sy) + 2;

		boxes.clear();
		boxes.reserve(t.LeafBounds.size() * 6);
		for (const AABB& leaf : t.LeafBounds)
		{
			int64_t v[6];
			if (!AxisSpan(leaf.Min.x, leaf.Max.x, g.G[0], dx, v[0], v[1]) || !AxisSpan(leaf.Min.y, leaf.Max.y, g.G[1], dy, v[2], v[3]) ||
				!AxisSpan(leaf.Min.z, leaf.Max.z, g.G[2], dz, v[4], v[5]))
			{
				error = "octree leaf outside the meshing lattice";
				return false;
			}
			boxes.insert(boxes.end(), v, v + 6);
		}
		return true;
	}

	cudaError_t Engine::Sodapop(const Program& p, const SodapopGrid& g, const std::vector<int64_t>& boxes, SodapopMesh& out,
		cudaStream_t s)
	{
		out = SodapopMesh();
		out.Grid = g;
		const int64_t lattice = (g.SX + 1) * (g.SY + 1) * g.LZ;
		const int64_t words = (g.Limit + 31) / 32;
		const int leaves = (int)(boxes.size() / 6);
		if (!HostCounts) TG_TRY(cudaMallocHost(&HostCounts, 8 * sizeof(uint32_t)));
		TG_TRY(LatticeBuf.Reserve((size_t)lattice * sizeof(float)));
		TG_TRY(Words.Reserve((size_t)words * 4));
		TG_TRY(WordBase.Reserve((size_t)words * 4));
		TG_TRY(Counts.Reserve(4 * sizeof(uint32_t)));
		TG_TRY(Scratch.Reserve(ScanScratchWords(words) * 4));
		TG_TRY(SodaCache.Reserve((size_t)g.Limit));
		TG_TRY(SodaBoxes.Reserve((boxes.empty() ? 1 : boxes.size()) * sizeof(int64_t)));
		if (!boxes.empty())
			TG_TRY(cudaMemcpyAsync(SodaBoxes.Ptr, boxes.data(), boxes.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s));

		Begin("soda_lattice", s);
		TG_TRY(LaunchSodapopLattice(p.View, g, LatticeBuf.As<float>(), s));
		End(s);
		Begin("soda_cache", s);
		TG_TRY(LaunchSodapopCache(SodaBoxes.As<int64_t>(), leaves, g, SodaCache.As<uint8_t>(), s));
		End(s);
		Begin("soda_flags", s);
		TG_TRY(LaunchSodapopFlags(LatticeBuf.As<float>(), SodaCache.As<uint8_t>(), g, Words.As<uint32_t>(), s));
		End(s);
		Begin("scan", s);
		TG_TRY(LaunchExclusiveScan(Words.As<uint32_t>(), words, true, WordBase.As<uint32_t>(), Counts.As<uint32_t>(), Scratch.As<uint32_t>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(HostCounts, Counts.Ptr, 4, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		const uint32_t vcount = HostCounts[0];

		TG_TRY(Vertices.Reserve((size_t)vcount * 12 + 12));
		TG_TRY(Cubes.Reserve((size_t)vcount * 4 + 4));
		TG_TRY(FaceCounts.Reserve((size_t)vcount * 4 + 4));
		TG_TRY(FaceBase.Reserve((size_t)vcount * 4 + 4));
		TG_TRY(Scratch.Reserve(ScanScratchWords(vcount) * 4));
		Begin("soda_vertices", s);
		TG_TRY(LaunchSodapopVertices(LatticeBuf.As<float>(), g, Words.As<uint32_t>(), WordBase.As<uint32_t>(), Vertices.As<float>(),
			Cubes.As<uint32_t>(), FaceCounts.As<uint32_t>(), s));
		End(s);
		Begin("scan", s);
		TG_TRY(LaunchExclusiveScan(FaceCounts.As<uint32_t>(), vcount, false, FaceBase.As<uint32_t>(), Counts.As<uint32_t>() + 1,
			Scratch.As<uint32_t>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(HostCounts + 1, Counts.As<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		const uint32_t fcount = HostCounts[1];

		TG_TRY(Faces.Reserve((size_t)fcount * 12 + 12));
		Begin("soda_faces", s);
		TG_TRY(LaunchSodapopFaces(LatticeBuf.As<float>(), g, Words.As<uint32_t>(), WordBase.As<uint32_t>(), Cubes.As<uint32_t>(),
			FaceBase.As<uint32_t>(), vcount, Faces.As<uint32_t>(), s));
		End(s);
		TG_TRY(Normals.Reserve((size_t)vcount * 12 + 12));
		TG_TRY(SodaColors.Reserve((size_t)vcount * 16 + 16));
		Begin("soda_attributes", s);
		TG_TRY(LaunchSodapopAttributes(p.View, Vertices.As<float>(), vcount, Normals.As<float>(), SodaColors.As<float>(), s));
		End(s);
		TG_TRY(cudaStreamSynchronize(s));
		Collect();
		out.VertexCount = vcount;
		out.FaceCount = fcount;
		out.Positions = Vertices.As<float>();
		out.Normals = Normals.As<float>();
		out.Colors = SodaColors.As<float>();
		out.Faces = Faces.As<uint32_t>();
		out.Cells = Cubes.As<uint32_t>();
		return cudaSuccess;
	}
}
