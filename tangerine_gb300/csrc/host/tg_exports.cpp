// Host side of the point-cloud export (export.cpp:384-480) and the MagicaVoxel export
// (magica.cpp:27-72): lattice planning, the kernel sequence of kernels/tg_exports.cu, and
// the .vox writer.
#include "tg_engine.hpp"

#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <unordered_map>

#define TG_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return _e; } while (0)

namespace tg
{
	bool CloudPlan(const float lo[3], const float hi[3], const float step[3], CloudSpec& s, std::string& error)
	{
		double total = 1.0;
		int32_t n[3];
		for (int a = 0; a < 3; ++a)
		{
			if (!(step[a] > 0.0f) || !std::isfinite(step[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
			{
				error = "point cloud bounds and step must be finite, the step positive";
				return false;
			}
			s.Start[a] = lo[a];
			s.Step[a] = step[a];
			// Half = Step / vec3(2.0)
			s.Half[a] = step[a] / 2.0f;
			// ivec3(ceil((Stop - Start) / Step))
			const float c = ceilf((hi[a] - lo[a]) / step[a]);
			if (!(c < 2147483648.0f)) { error = "point cloud lattice too large"; return false; }
			n[a] = c > 0.0f ? (int32_t)c : 0;
			total *= (double)n[a];
		}
		if (total >= 2147483648.0)
		{
			error = "point cloud lattice has more voxels than the reference's int cell numbers hold";
			return false;
		}
		s.IX = n[0]; s.IY = n[1]; s.IZ = n[2];
		s.Total = (int64_t)n[0] * n[1] * n[2];
		// length(Half) = sqrt(dot(Half, Half))
		s.Diagonal = sqrtf((s.Half[0] * s.Half[0] + s.Half[1] * s.Half[1]) + s.Half[2] * s.Half[2]);
		return true;
	}

	bool VoxPlan(const AABB& b, float grid_size, VoxSpec& s, std::string& error)
	{
		if (!std::isfinite(grid_size) || !(grid_size > 0.0f))
		{
			error = "voxel grid size must be positive";
			return false;
		}
		double total = 1.0;
		const float lo[3] = { b.Min.x, b.Min.y, b.Min.z }, hi[3] = { b.Max.x, b.Max.y, b.Max.z };
		int32_t n[3];
		for (int a = 0; a < 3; ++a)
		{
			// ivec3(glm::ceil(Max - Min) * GridSize)
			const float c = ceilf(hi[a] - lo[a]) * grid_size;
			if (!(c < 2147483648.0f) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
			{
				error = "voxel lattice too large or unbounded";
				return false;
			}
			n[a] = c > 0.0f ? (int32_t)c : 0;
			total *= (double)n[a];
			s.Min[a] = lo[a];
			s.Max[a] = hi[a];
		}
		if (total >= 2147483648.0)
		{
			error = "voxel lattice has more voxels than the reference's int cell numbers hold";
			return false;
		}
		s.SX = n[0]; s.SY = n[1]; s.SZ = n[2];
		s.Total = (int64_t)n[0] * n[1] * n[2];
		// Radius = distance(Min, mix(Min, Max, vec3(.5) / vec3(Size))), mix = x * (1 - a) + y * a
		float d[3];
		for (int a = 0; a < 3; ++a)
		{
			const float alpha = 0.5f / (float)n[a];
			const float m = lo[a] * (1.0f - alpha) + hi[a] * alpha;
			d[a] = m - lo[a];
		}
		s.Radius = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
		return true;
	}

	cudaError_t Engine::PointCloud(const Program& p, const CloudSpec& s, int refine, bool attributes, DeviceMesh& out, cudaStream_t st,
		const ExportOptions* control)
	{
		out = DeviceMesh();
		const int64_t words = (s.Total + 31) / 32;
		if (!HostCounts) TG_TRY(cudaMallocHost(&HostCounts, 8 * sizeof(uint32_t)));
		TG_TRY(Words.Reserve((size_t)(words ? words : 1) * 4));
		TG_TRY(WordBase.Reserve((size_t)(words ? words : 1) * 4));
		TG_TRY(Counts.Reserve(4 * sizeof(uint32_t)));
		TG_TRY(Scratch.Reserve(ScanScratchWords(words) * 4 + 4));
		PreValid = false;   // these bits replace a pending PreClassify's
		TG_TRY(BrickBits.Reserve(VoxelBrickWords(s.IX, s.IY, s.IZ) * 4));
		Begin("cloud_flags", st);
		TG_TRY(LaunchCloudFlags(p.View, s, BrickBits.As<uint32_t>(), Words.As<uint32_t>(), st));
		End(st);
		// The kept voxels' numbers in increasing order (bitmask -> scan -> list).
		TG_TRY(Cubes.Reserve((size_t)(words ? words : 1) * 32 * 4));
		Begin("list_cells", st);
		TG_TRY(LaunchListBricks(Words.As<uint32_t>(), s.Total, WordBase.As<uint32_t>(), Scratch.As<uint32_t>(), Cubes.As<uint32_t>(),
			Counts.As<uint32_t>(), st));
		End(st);
		TG_TRY(cudaMemcpyAsync(HostCounts, Counts.Ptr, 4, cudaMemcpyDeviceToHost, st));
		TG_TRY(cudaStreamSynchronize(st));
		const uint32_t n = HostCounts[0];
		if (control)
		{
			// End of the voxel search (PointCloudExportThread's ExportState.store(2)).
			if (control->Progress) control->Progress->store(1.0f);
			if (control->Stage) control->Stage->store(2);
			if (control->Active && !control->Active->load())
			{
				if (control->Cancelled) *control->Cancelled = true;
				Collect();
				return cudaSuccess;
			}
			if (control->Stage && control->Stage->load() > 2) refine = 0;
		}
		TG_TRY(Vertices.Reserve((size_t)n * 12 + 12));
		Begin("cloud_refine", st);
		TG_TRY(LaunchCloudRefine(p.View, s, Cubes.As<uint32_t>(), Counts.As<uint32_t>(), n, refine, Vertices.As<float>(), st));
		End(st);
		out.VertexCount = n;
		out.Vertices = Vertices.As<float>();
		out.Cubes = Cubes.As<uint32_t>();
		if (attributes)
		{
			TG_TRY(Normals.Reserve((size_t)n * 12 + 12));
			uint8_t* colors = nullptr;
			if (p.Host.Header.HasPaint)
			{
				TG_TRY(Colors.Reserve((size_t)n * 3 + 3));
				colors = Colors.As<uint8_t>();
			}
			Begin("attributes", st);
			TG_TRY(LaunchVertexAttributes(p.View, Vertices.As<float>(), n, Normals.As<float>(), colors, st));
			End(st);
			out.Normals = Normals.As<float>();
			out.Colors = colors;
		}
		TG_TRY(cudaStreamSynchronize(st));
		Collect();
		return cudaSuccess;
	}

	cudaError_t Engine::Voxels(const Program& p, const VoxSpec& s, std::vector<uint32_t>& cells, cudaStream_t st)
	{
		cells.clear();
		const int64_t words = (s.Total + 31) / 32;
		if (!HostCounts) TG_TRY(cudaMallocHost(&HostCounts, 8 * sizeof(uint32_t)));
		TG_TRY(Words.Reserve((size_t)(words ? words : 1) * 4));
		TG_TRY(WordBase.Reserve((size_t)(words ? words : 1) * 4));
		TG_TRY(Counts.Reserve(4 * sizeof(uint32_t)));
		TG_TRY(Scratch.Reserve(ScanScratchWords(words) * 4 + 4));
		TG_TRY(Cubes.Reserve((size_t)(words ? words : 1) * 32 * 4));
		PreValid = false;   // these bits replace a pending PreClassify's
		TG_TRY(BrickBits.Reserve(VoxelBrickWords(s.SX, s.SY, s.SZ) * 4));
		Begin("vox_flags", st);
		TG_TRY(LaunchVoxFlags(p.View, s, BrickBits.As<uint32_t>(), Words.As<uint32_t>(), st));
		End(st);
		Begin("list_cells", st);
		TG_TRY(LaunchListBricks(Words.As<uint32_t>(), s.Total, WordBase.As<uint32_t>(), Scratch.As<uint32_t>(), Cubes.As<uint32_t>(),
			Counts.As<uint32_t>(), st));
		End(st);
		TG_TRY(cudaMemcpyAsync(HostCounts, Counts.Ptr, 4, cudaMemcpyDeviceToHost, st));
		TG_TRY(cudaStreamSynchronize(st));
		const uint32_t n = HostCounts[0];
		cells.resize(n);
		if (n) TG_TRY(cudaMemcpyAsync(cells.data(), Cubes.Ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
		TG_TRY(cudaStreamSynchronize(st));
		Collect();
		return cudaSuccess;
	}

	// ---- MagicaVoxel file ---------------------------------------------------------------
	//
	// The layout VoxWriter produces (voxwriter/VoxWriter.cpp): "VOX " 150, a MAIN chunk whose
	// children are, per cube of at most M = clamp(limit, 0, 126) voxels a side in the order
	// cubes were first touched, a SIZE chunk (M+1 per axis) and an XYZI chunk (the voxels'
	// x%M, y%M, z%M, colour in insertion order); then the scene graph: a root transform
	// (node 0) over a group (node 1) whose children are one transform (node 2+2i, layer 0,
	// frame attribute "_t" = the cube's translation) over one shape (node 3+2i, model i) per
	// cube.  No palette chunk: VoxExport adds no colours.  Every chunk is id, content bytes,
	// children bytes (0 except MAIN), content.
	namespace
	{
		struct VoxBytes
		{
			std::vector<uint8_t> B;
			void I32(int32_t v)
			{
				const uint32_t u = (uint32_t)v;
				B.push_back((uint8_t)(u & 0xFFu));
				B.push_back((uint8_t)((u >> 8) & 0xFFu));
				B.push_back((uint8_t)((u >> 16) & 0xFFu));
				B.push_back((uint8_t)((u >> 24) & 0xFFu));
			}
			void Id(const char* s) { for (int i = 0; i < 4; ++i) B.push_back((uint8_t)s[i]); }
			void Str(const std::string& s) { I32((int32_t)s.size()); B.insert(B.end(), s.begin(), s.end()); }
			void Chunk(const char* id, int32_t content) { Id(id); I32(content); I32(0); }
		};

		struct Cube
		{
			int32_t Ox, Oy, Oz;
			std::vector<uint8_t> Voxels;
		};
	}

	bool WriteVoxFile(const std::string& path, const int32_t size[3], const int32_t* xyzc, size_t count)
	{
		// ct::clamp<int32_t>(limit, 0, 126)
		int32_t M[3];
		for (int a = 0; a < 3; ++a) M[a] = size[a] < 0 ? 0 : (size[a] > 126 ? 126 : size[a]);
		std::vector<Cube> cubes;
		std::unordered_map<int64_t, int32_t> cubeOf;   // packed cube coordinates -> cube number
		int32_t minX = 10000000, minY = 10000000, minZ = 10000000;
		double lower[3] = { 1e7, 1e7, 1e7 }, upper[3] = { 0.0, 0.0, 0.0 };
		for (size_t v = 0; v < count; ++v)
		{
			const int32_t x = xyzc[v * 4], y = xyzc[v * 4 + 1], z = xyzc[v * 4 + 2];
			const uint8_t c = (uint8_t)xyzc[v * 4 + 3];
			if (M[0] == 0 || M[1] == 0 || M[2] == 0) return false;
			const int32_t ox = (int32_t)std::floor((double)x / (double)M[0]);
			const int32_t oy = (int32_t)std::floor((double)y / (double)M[1]);
			const int32_t oz = (int32_t)std::floor((double)z / (double)M[2]);
			// VoxWriter::AddVoxel updates the minima this way: y and z take min(minCubeX, o).
			minX = minX < ox ? minX : ox;
			minY = minX < oy ? minX : oy;
			minZ = minX < oz ? minX : oz;
			const int64_t key = ((int64_t)(ox & 0x1FFFFF) << 42) | ((int64_t)(oy & 0x1FFFFF) << 21) | (int64_t)(oz & 0x1FFFFF);
			auto it = cubeOf.find(key);
			int32_t ci;
			if (it == cubeOf.end())
			{
				ci = (int32_t)cubes.size();
				cubeOf.emplace(key, ci);
				cubes.push_back(Cube{ ox, oy, oz, {} });
			}
			else ci = it->second;
			const double pt[3] = { (double)x, (double)y, (double)z };
			for (int a = 0; a < 3; ++a)
			{
				lower[a] = lower[a] < pt[a] ? lower[a] : pt[a];
				upper[a] = upper[a] > pt[a] ? upper[a] : pt[a];
			}
			// VoxExport adds each voxel once, so no voxel is merged twice.
			Cube& cb = cubes[(size_t)ci];
			cb.Voxels.push_back((uint8_t)(x % M[0]));
			cb.Voxels.push_back((uint8_t)(y % M[1]));
			cb.Voxels.push_back((uint8_t)(z % M[2]));
			cb.Voxels.push_back(c);
		}
		VoxBytes f;
		f.Id("VOX ");
		f.I32(150);
		f.Id("MAIN");
		f.I32(0);
		const size_t childSizeAt = f.B.size();
		f.I32(0);
		const size_t header = f.B.size();
		const int32_t count32 = (int32_t)cubes.size();
		std::vector<std::string> translations;
		for (const Cube& c : cubes)
		{
			f.Chunk("SIZE", 12);
			f.I32(M[0] + 1); f.I32(M[1] + 1); f.I32(M[2] + 1);
			const int32_t nv = (int32_t)(c.Voxels.size() / 4);
			f.Chunk("XYZI", 4 * (1 + nv));
			f.I32(nv);
			f.B.insert(f.B.end(), c.Voxels.begin(), c.Voxels.end());
			// (cube - min + 0.5f) * M in float, then the volume's lower bound and half its
			// size in double (x, y); z without the volume terms, floored in float.
			const double sx = upper[0] - lower[0], sy = upper[1] - lower[1];
			const float fx = ((float)(c.Ox - minX) + 0.5f) * (float)M[0];
			const float fy = ((float)(c.Oy - minY) + 0.5f) * (float)M[1];
			const float fz = ((float)(c.Oz - minZ) + 0.5f) * (float)M[2];
			const int tx = (int)std::floor((double)fx - lower[0] - sx * 0.5);
			const int ty = (int)std::floor((double)fy - lower[1] - sy * 0.5);
			const int tz = (int)std::floor(fz);
			translations.push_back(std::to_string(tx) + " " + std::to_string(ty) + " " + std::to_string(tz));
		}
		// Root transform: node 0 -> node 1, no layer, one empty frame.
		f.Chunk("nTRN", 4 * 5 + 4 + 4);
		f.I32(0); f.I32(0); f.I32(1); f.I32(-1); f.I32(-1); f.I32(1); f.I32(0);
		// Group: node 1 with the cubes' transforms as children.
		f.Chunk("nGRP", 4 * (2 + count32) + 4);
		f.I32(1); f.I32(0); f.I32(count32);
		for (int32_t i = 0; i < count32; ++i) f.I32(2 + 2 * i);
		for (int32_t i = 0; i < count32; ++i)
		{
			const std::string& t = translations[(size_t)i];
			const int32_t frame = 4 + (4 + 2) + (4 + (int32_t)t.size());
			f.Chunk("nTRN", 4 * 5 + 4 + frame);
			f.I32(2 + 2 * i); f.I32(0); f.I32(3 + 2 * i); f.I32(-1); f.I32(0); f.I32(1);
			f.I32(1); f.Str("_t"); f.Str(t);
			f.Chunk("nSHP", 4 * 2 + 4 + 8);
			f.I32(3 + 2 * i); f.I32(0); f.I32(1); f.I32(i); f.I32(0);
		}
		const uint32_t children = (uint32_t)(f.B.size() - header);
		for (int k = 0; k < 4; ++k) f.B[childSizeAt + k] = (uint8_t)((children >> (8 * k)) & 0xFFu);
		FILE* out = std::fopen(path.c_str(), "wb");
		if (!out) return false;
		const bool ok = std::fwrite(f.B.data(), 1, f.B.size(), out) == f.B.size();
		return std::fclose(out) == 0 && ok;
	}
}
