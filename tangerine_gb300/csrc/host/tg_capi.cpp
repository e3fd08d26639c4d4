// The C ABI (include/tangerine_gb300.h): Tangerine's tree API re-enabled over
// reference-counted trees, and the GPU-native tg_* entry points.
#include "../../../include/tangerine_gb300.h"

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "tg_engine.hpp"
#include "tg_surrogate.hpp"
#include "tg_batch.hpp"
#include "tg_octree.hpp"
#include "tg_tree.hpp"

using namespace tg;

namespace
{
	Node* AsNode(void* h) { return static_cast<Node*>(h); }
	NodeRef Borrow(void* h) { return NodeRef::Share(AsNode(h)); }     // caller keeps its reference
	NodeRef Adopt(void* h) { return NodeRef(AsNode(h)); }             // take over the caller's reference
	void* Hand(NodeRef r) { return r.release(); }

	tg_status CudaFail(cudaError_t e, const char* what)
	{
		SetError(std::string(what) + ": " + cudaGetErrorString(e));
		return TG_ERR_CUDA;
	}

	cudaStream_t StreamOf(void* s) { return s ? static_cast<cudaStream_t>(s) : Engine::Get().DefaultStream(); }

	bool ToGridSpec(const tg_grid* g, GridSpec& out)
	{
		const float dy = g && g->step_y != 0.0f ? g->step_y : (g ? g->step : 0.0f);
		const float dz = g && g->step_z != 0.0f ? g->step_z : (g ? g->step : 0.0f);
		if (!g || g->nx < 2 || g->ny < 2 || g->nz < 2 || !(g->step > 0.0f) || !(dy > 0.0f) || !(dz > 0.0f) ||
			!std::isfinite(g->step) || !std::isfinite(dy) || !std::isfinite(dz))
		{
			SetError("a lattice needs at least 2 points per axis and a positive step");
			return false;
		}
		if (g->nx > (1 << 20) || g->ny > (1 << 20) || g->nz > (1 << 20) ||
			(double)(g->nx - 1) * (double)(g->ny - 1) * (double)(g->nz - 1) >= 4294967296.0)
		{
			SetError("lattice too large: cube indices must fit in 32 bits");
			return false;
		}
		out = GridSpec{ g->x0, g->y0, g->z0, g->step, dy, dz, (int)g->nx, (int)g->ny, (int)g->nz };
		return true;
	}

	// MeshExportThread's lattice (export.cpp:324-337): ModelMin -= Step * 2, then
	// ceil((ModelMax - ModelMin) / Step) cells per axis.
	void ExportLattice(Vec3 lo, Vec3 hi, Vec3 step, tg_grid& g)
	{
		lo = lo - step * Vec3(2.0f);
		const Vec3 span = hi - lo;
		const Vec3 ext(span.x / step.x, span.y / step.y, span.z / step.z);
		g.x0 = lo.x; g.y0 = lo.y; g.z0 = lo.z;
		g.step = step.x;
		g.step_y = step.y;
		g.step_z = step.z;
		g.nx = (int64_t)std::ceil(ext.x) + 1;
		g.ny = (int64_t)std::ceil(ext.y) + 1;
		g.nz = (int64_t)std::ceil(ext.z) + 1;
	}

	// An export run with ExportOptions::Host: its host blocks become the tg_mesh.
	tg_status TakeHostMesh(cudaError_t e, HostMeshOut& h, tg_mesh* out, const char* what)
	{
		std::memset(out, 0, sizeof *out);
		if (e == cudaErrorLaunchTimeout)
		{
			// A bounded device wait ran out; the engine said which.
			FreeHostMesh(h);
			SetError(std::string(what) + ": " + LastError());
			return TG_ERR_CUDA;
		}
		if (e != cudaSuccess)
		{
			FreeHostMesh(h);
			return CudaFail(e, what);
		}
		if (h.OutOfMemory)
		{
			SetError("out of host memory for the mesh");
			return TG_ERR_MEMORY;
		}
		out->vertex_count = h.VertexCount;
		out->face_count = h.FaceCount;
		out->vertices = h.Vertices;
		out->normals = h.Normals;
		out->colors = h.Colors;
		out->faces = h.Faces;
		out->cubes = h.Cubes;
		return TG_OK;
	}

	tg_status CopyMeshToHost(const DeviceMesh& dm, tg_mesh* out, cudaStream_t s)
	{
		std::memset(out, 0, sizeof *out);
		out->vertex_count = dm.VertexCount;
		out->face_count = dm.FaceCount;
		const size_t v = dm.VertexCount ? dm.VertexCount : 1, f = dm.FaceCount ? dm.FaceCount : 1;
		auto take = [](size_t bytes) -> void*
		{
			void* p = HostPool::Get().Take(bytes);
			return p ? p : std::malloc(bytes);
		};
		out->vertices = (float*)take(v * 12);
		out->normals = (float*)take(v * 12);
		out->faces = (uint32_t*)take(f * 12);
		out->cubes = (uint32_t*)take(v * 4);
		out->colors = dm.Colors ? (uint8_t*)take(v * 3) : nullptr;
		if (!out->vertices || !out->normals || !out->faces || !out->cubes || (dm.Colors && !out->colors))
		{
			tg_mesh_free(out);
			SetError("out of host memory for the mesh");
			return TG_ERR_MEMORY;
		}
		cudaError_t e = cudaSuccess;
		if (dm.VertexCount)
		{
			e = cudaMemcpyAsync(out->vertices, dm.Vertices, dm.VertexCount * 12, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess && dm.Normals) e = cudaMemcpyAsync(out->normals, dm.Normals, dm.VertexCount * 12, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaMemcpyAsync(out->cubes, dm.Cubes, dm.VertexCount * 4, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess && dm.Colors) e = cudaMemcpyAsync(out->colors, dm.Colors, dm.VertexCount * 3, cudaMemcpyDeviceToHost, s);
		}
		if (e == cudaSuccess && dm.FaceCount) e = cudaMemcpyAsync(out->faces, dm.Faces, dm.FaceCount * 12, cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		if (e != cudaSuccess)
		{
			tg_mesh_free(out);
			return CudaFail(e, "copying the mesh to the host");
		}
		if (!dm.Normals) std::memset(out->normals, 0, v * 12);
		return TG_OK;
	}

	ExportOptions OptionsOf(uint32_t flags)
	{
		ExportOptions o;
		o.Attributes = (flags & TG_MESH_ATTRIBUTES) != 0;
		o.Dense = (flags & TG_MESH_DENSE) != 0;
		const int b = (int)((flags >> 8) & 0xFFu);
		o.BrickSize = b == 0 ? 7 : b;
		const int lanes = (int)((flags >> 16) & 0xFu);
		// Default: 2 points per thread for the culled export, 4 for the dense one (measured).
		o.Lanes = (lanes == 1 || lanes == 2 || lanes == 4) ? lanes : (o.Dense ? 4 : 2);
		o.Staged = (flags & TG_MESH_STAGED) != 0;
		return o;
	}

	tg_status CompileInto(void* tree, std::unique_ptr<tg_program>& prog)
	{
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		prog.reset(new (std::nothrow) tg_program());
		if (!prog) { SetError("out of host memory"); return TG_ERR_MEMORY; }
		std::string err;
		if (!CompileTree(Borrow(tree), prog->Host, err))
		{
			SetError(err);
			return TG_ERR_UNBOUNDED;
		}
		cudaError_t e = Engine::Get().Upload(*prog);
		if (e != cudaSuccess) return CudaFail(e, "uploading the program");
		return TG_OK;
	}

	void WriteFileError(const char* path) { SetError(std::string("cannot write ") + (path ? path : "(null)")); }

	// The asynchronous export behind MeshExport: one job at a time on a detached thread,
	// with the reference's progress words and flags (export.cpp:48-57) -- Active is
	// ExportActive, Stage ExportState -- and the job's outcome for tg_export_result.  Never
	// destroyed, so a job still running at process exit touches no destroyed state.
	struct ExportJob
	{
		std::mutex M;
		std::condition_variable CV;
		bool Running = false;
		tg_status Result = TG_OK;
		std::string Error;
		std::atomic<bool> Active{ false };
		std::atomic<int> Stage{ 0 };
		std::atomic<float> Generation{ 0.0f }, Refinement{ 0.0f }, Secondary{ 0.0f }, Write{ 0.0f };
		int PauseAt = 0;            // test hook (tg_debug_export_pause)
		bool Paused = false;
	};

	ExportJob& Job()
	{
		static ExportJob* j = new ExportJob();
		return *j;
	}

	struct ExportArgs
	{
		NodeRef Tree;
		std::string Path;
		float Lo[3], Hi[3], Step[3];
		int Refine = 0, Format = 1;
		bool PointCloud = false;
		float Scale = 1.0f;
	};

	// The test hook's wait at the start of `stage`.
	void PauseAt(ExportJob& j, int stage)
	{
		std::unique_lock<std::mutex> l(j.M);
		if (j.PauseAt != stage) return;
		j.Paused = true;
		j.CV.notify_all();
		j.CV.wait_for(l, std::chrono::seconds(30), [&]() { return j.PauseAt != stage || !j.Active.load(); });
		j.Paused = false;
	}

	// MeshExportThread / PointCloudExportThread (export.cpp:320-480) on the GPU: stage 1
	// builds the octree, compiles and runs the export (or the voxel search), stage 2 the
	// point cloud's refinement, stage 3 writes the file; stage 0 when done.  Halting stops at
	// the next phase boundary and writes no file.
	void RunExportJob(ExportArgs a)
	{
		ExportJob& j = Job();
		tg_status st = TG_OK;
		std::string err;
		bool cancelled = false;
		tg_mesh m;
		std::memset(&m, 0, sizeof m);
		bool haveMesh = false;
		std::unique_ptr<tg_program> prog;
		PauseAt(j, 1);
		if (!j.Active.load()) cancelled = true;
		else if ((st = CompileInto(a.Tree.get(), prog)) != TG_OK) err = LastError();
		if (st == TG_OK && !cancelled)
		{
			Engine& eng = Engine::Get();
			ExportOptions control = OptionsOf(TG_MESH_ATTRIBUTES);
			control.Active = &j.Active;
			control.Cancelled = &cancelled;
			control.Stage = &j.Stage;
			control.Progress = &j.Generation;
			if (a.PointCloud)
			{
				CloudSpec cs;
				if (!CloudPlan(a.Lo, a.Hi, a.Step, cs, err)) st = TG_ERR_UNSUPPORTED;
				else
				{
					std::lock_guard<std::mutex> lock(eng.Mutex);
					const cudaStream_t s = eng.DefaultStream();
					DeviceMesh dm;
					const cudaError_t e = eng.PointCloud(*prog, cs, a.Refine, true, dm, s, &control);
					if (e != cudaSuccess) { st = CudaFail(e, "exporting the point cloud"); err = LastError(); }
					else if (!cancelled)
					{
						j.Refinement.store(1.0f);
						st = CopyMeshToHost(dm, &m, s);
						if (st == TG_OK) haveMesh = true;
						else err = LastError();
					}
				}
			}
			else
			{
				tg_grid g;
				GridSpec gs;
				if (tg_export_grid_axes(a.Lo, a.Hi, a.Step, &g) != TG_OK || !ToGridSpec(&g, gs))
				{
					st = TG_ERR_INVALID;
					err = LastError();
				}
				else
				{
					HostMeshOut host;
					control.Host = &host;
					DeviceMesh dm;
					cudaError_t e;
					{
						std::lock_guard<std::mutex> lock(eng.Mutex);
						e = eng.Export(*prog, gs, control, dm, eng.DefaultStream());
					}
					if (cancelled && e == cudaSuccess) FreeHostMesh(host);
					else
					{
						st = TakeHostMesh(e, host, &m, "exporting the mesh");
						if (st == TG_OK) haveMesh = true;
						else err = LastError();
					}
				}
			}
		}
		if (st == TG_OK && !cancelled)
		{
			// ExportState.store(2), then (3): normals and colours came with the mesh.
			if (!a.PointCloud) j.Stage.store(2);
			j.Stage.store(3);
			j.Secondary.store(1.0f);
			PauseAt(j, 3);
			if (!j.Active.load()) cancelled = true;
		}
		if (st == TG_OK && !cancelled)
		{
			st = a.Format == 1 ? tg_write_ply(&m, a.Path.c_str(), a.Scale) : tg_write_stl(prog.get(), &m, a.Path.c_str(), a.Scale, nullptr);
			if (st != TG_OK) err = LastError();
			else if (!j.Active.load())
			{
				cancelled = true;
				std::remove(a.Path.c_str());
			}
			else j.Write.store(1.0f);
		}
		if (haveMesh) tg_mesh_free(&m);
		prog.reset();
		a.Tree = NodeRef();
		if (cancelled && st == TG_OK)
		{
			st = TG_ERR_CANCELLED;
			err = "the export was halted (CancelExport(true))";
		}
		{
			std::lock_guard<std::mutex> l(j.M);
			j.Result = st;
			j.Error = err;
			j.Running = false;
			j.Paused = false;
			j.Stage.store(0);
		}
		j.CV.notify_all();
	}

	// An octree's cells in the oracle's dump layout (tg_debug_octree).
	int64_t DumpOctree(const Octree& o, float* cells, int32_t* children, int64_t cell_capacity, uint32_t* words,
		int64_t word_capacity, int64_t* word_count);
}

extern "C"
{
	// ---- tree API (tangerine/c_sdf.cpp) -------------------------------------------------
	TANGERINE_API float EvalTree(void* h, float x, float y, float z)
	{
		return AsNode(h)->Eval(Vec3(x, y, z));
	}

	TANGERINE_API void* ClipTree(void* h, float x, float y, float z, float radius)
	{
		const Vec3 p(x, y, z);
		NodeRef clipped = AsNode(h)->Clip(p, radius);
		if (clipped && std::fabs(clipped->Eval(p)) > radius) return nullptr;
		return Hand(std::move(clipped));
	}

	TANGERINE_API ::RayHit RayMarchTree(void* h, float sx, float sy, float sz, float dx, float dy, float dz, int iters, float eps)
	{
		const tg::RayHit r = RayMarch(*AsNode(h), Vec3(sx, sy, sz), Vec3(dx, dy, dz), iters, eps);
		::RayHit out;
		out.Hit = r.Hit;
		out.Travel = r.Travel;
		out.Position[0] = r.Position.x;
		out.Position[1] = r.Position.y;
		out.Position[2] = r.Position.z;
		return out;
	}

	TANGERINE_API void DiscardTree(void* h) { if (h) Adopt(h); }
	TANGERINE_API bool TreeHasFiniteBounds(void* h) { return AsNode(h)->HasFiniteBounds(); }
	TANGERINE_API void MoveTree(void* h, float x, float y, float z) { AsNode(h)->Move(Vec3(x, y, z)); }
	TANGERINE_API void RotateTree(void* h, float x, float y, float z, float w) { AsNode(h)->Rotate(Quat{ w, x, y, z }); }
	TANGERINE_API void AlignTree(void* h, float x, float y, float z) { SDF::Align(*AsNode(h), Vec3(x, y, z)); }
	TANGERINE_API void ScaleTree(void* h, float s) { AsNode(h)->Scale(s); }

	TANGERINE_API void PaintTree(float r, float g, float b, void* h)
	{
		auto m = std::make_shared<Material>();
		m->Rgb[0] = r; m->Rgb[1] = g; m->Rgb[2] = b;
		AsNode(h)->ApplyMaterial(m, false);
	}

	TANGERINE_API void PaintOverTree(float r, float g, float b, void* h)
	{
		auto m = std::make_shared<Material>();
		m->Rgb[0] = r; m->Rgb[1] = g; m->Rgb[2] = b;
		AsNode(h)->ApplyMaterial(m, true);
	}

	TANGERINE_API void* CopyTree(void* h) { return h ? Hand(tg::CopyTree(*AsNode(h))) : nullptr; }
	TANGERINE_API void GradientTree(void* h, float x, float y, float z, float* out)
	{
		const Vec3 g = AsNode(h)->Gradient(Vec3(x, y, z));
		out[0] = g.x; out[1] = g.y; out[2] = g.z;
	}
	TANGERINE_API void RotateTreeX(void* h, float degrees) { SDF::RotateX(*AsNode(h), degrees); }
	TANGERINE_API void RotateTreeY(void* h, float degrees) { SDF::RotateY(*AsNode(h), degrees); }
	TANGERINE_API void RotateTreeZ(void* h, float degrees) { SDF::RotateZ(*AsNode(h), degrees); }

	TANGERINE_API int64_t tg_tree_spec(void* h, float* out, int64_t capacity)
	{
		if (!h) { SetError("null tree handle"); return -1; }
		std::vector<float> spec;
		tg::WriteSpec(*AsNode(h), spec);
		if (out)
			for (int64_t i = 0; i < capacity && i < (int64_t)spec.size(); ++i) out[i] = spec[(size_t)i];
		return (int64_t)spec.size();
	}

	TANGERINE_API void* MakeSphereBrush(float r) { return Hand(SDF::Sphere(r)); }
	TANGERINE_API void* MakeEllipsoidBrush(float x, float y, float z) { return Hand(SDF::Ellipsoid(x, y, z)); }
	TANGERINE_API void* MakeBoxBrush(float x, float y, float z) { return Hand(SDF::Box(x, y, z)); }
	TANGERINE_API void* MakeTorusBrush(float major, float minor) { return Hand(SDF::Torus(major, minor)); }
	TANGERINE_API void* MakeCylinderBrush(float r, float e) { return Hand(SDF::Cylinder(r, e)); }
	TANGERINE_API void* MakePlaneOperand(float x, float y, float z) { return Hand(SDF::Plane(x, y, z)); }
	TANGERINE_API void* MakeConeBrush(float r, float h) { return Hand(SDF::Cone(r, h)); }
	TANGERINE_API void* MakeConinderBrush(float rl, float rh, float h) { return Hand(SDF::Coninder(rl, rh, h)); }

	TANGERINE_API void* MakeUnionOp(void* l, void* r) { return Hand(SDF::Union(Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeDiffOp(void* l, void* r) { return Hand(SDF::Diff(Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeInterOp(void* l, void* r) { return Hand(SDF::Inter(Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeBlendUnionOp(float k, void* l, void* r) { return Hand(SDF::BlendUnion(k, Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeBlendDiffOp(float k, void* l, void* r) { return Hand(SDF::BlendDiff(k, Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeBlendInterOp(float k, void* l, void* r) { return Hand(SDF::BlendInter(k, Adopt(l), Adopt(r))); }
	TANGERINE_API void* MakeFlateOp(void* h, float r) { return Hand(SDF::Flate(Adopt(h), r)); }

	TANGERINE_API void* MakeStencilOp(void* h, void* mask, float r, float g, float b, bool negative)
	{
		auto m = std::make_shared<Material>();
		m->Rgb[0] = r; m->Rgb[1] = g; m->Rgb[2] = b;
		return Hand(SDF::Stencil(Adopt(h), Adopt(mask), m, negative));
	}

	TANGERINE_API void* BuildTreeFromSpec(const float* spec, int count)
	{
		if (!spec || count <= 0) { SetError("empty tree spec"); return nullptr; }
		const char* err = nullptr;
		NodeRef t = BuildFromSpec(spec, count, &err);
		if (!t) { SetError(err ? err : "malformed tree spec"); return nullptr; }
		return Hand(std::move(t));
	}

	// ---- GPU-native API ------------------------------------------------------------------
	TANGERINE_API tg_status tg_compile(void* tree, tg_program** out)
	{
		if (!out) { SetError("null output"); return TG_ERR_INVALID; }
		*out = nullptr;
		std::unique_ptr<tg_program> prog;
		std::lock_guard<std::mutex> lock(Engine::Get().Mutex);
		const tg_status st = CompileInto(tree, prog);
		if (st == TG_OK) *out = prog.release();
		return st;
	}

	TANGERINE_API void tg_program_free(tg_program* p) { delete p; }

	TANGERINE_API tg_status tg_program_get_info(const tg_program* p, tg_program_info* out)
	{
		if (!p || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		out->octree_cells = p->Host.Header.NodeCount;
		out->code_quads = p->Host.Header.CodeQuads;
		out->materials = p->Host.Header.MaterialCount;
		out->has_paint = p->Host.Header.HasPaint;
		out->max_stack = p->Host.Header.MaxStack;
		out->bounds_min[0] = p->Host.Bounds.Min.x; out->bounds_min[1] = p->Host.Bounds.Min.y; out->bounds_min[2] = p->Host.Bounds.Min.z;
		out->bounds_max[0] = p->Host.Bounds.Max.x; out->bounds_max[1] = p->Host.Bounds.Max.y; out->bounds_max[2] = p->Host.Bounds.Max.z;
		out->compile_seconds = p->Host.BuildSeconds;
		out->distance_quads = p->Host.DistanceQuadsTotal;
		return TG_OK;
	}

	TANGERINE_API int64_t tg_tree_reference_words(void* tree, uint32_t* out, int64_t capacity)
	{
		if (!tree) return 0;
		const std::vector<uint32_t> w = CompileReferenceWords(*AsNode(tree));
		for (int64_t i = 0; i < (int64_t)w.size() && i < capacity; ++i) out[i] = w[i];
		return (int64_t)w.size();
	}

	TANGERINE_API int64_t tg_debug_octree(void* tree, float* cells, int32_t* children, int64_t cell_capacity,
		uint32_t* words, int64_t word_capacity, int64_t* word_count)
	{
		if (!tree) return -1;
		Octree o;
		if (!o.Build(Borrow(tree))) return -1;
		return DumpOctree(o, cells, children, cell_capacity, words, word_capacity, word_count);
	}

	TANGERINE_API int64_t tg_debug_meshing_octree(void* tree, float* cells, int32_t* children, int64_t cell_capacity,
		uint32_t* words, int64_t word_capacity, int64_t* word_count)
	{
		if (!tree) return -1;
		Octree o;
		if (!o.BuildMeshing(Borrow(tree))) return -1;
		return DumpOctree(o, cells, children, cell_capacity, words, word_capacity, word_count);
	}

	TANGERINE_API tg_status tg_debug_compile_seconds(void* tree, int meshing, double* octree_seconds, double* total_seconds)
	{
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		CompiledTree t;
		std::string err;
		if (!CompileTree(Borrow(tree), t, err, meshing ? OctreeKind::Meshing : OctreeKind::Export)) { SetError(err); return TG_ERR_UNBOUNDED; }
		if (octree_seconds) *octree_seconds = t.OctreeSeconds;
		if (total_seconds) *total_seconds = t.BuildSeconds;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_debug_root_program_check(void* tree, int64_t* code_quads, int32_t* stack_size)
	{
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		RootProgram seen;
		bool called = false;
		const RootHook hook = [&](const RootProgram& r) { seen = r; called = true; };
		CompiledTree t;
		std::string err;
		if (!CompileTree(Borrow(tree), t, err, OctreeKind::Export, &hook)) { SetError(err); return TG_ERR_UNBOUNDED; }
		if (!called) { SetError("no root program was handed out"); return TG_ERR_INVALID; }
		const OctNode& n0 = t.Nodes[0];
		std::vector<float> image(t.CodeFloats);
		t.CopyCode(image.data());
		const size_t from = (size_t)n0.DistanceCode * 4, to = (size_t)n0.SurfaceCode * 4;
		const bool samePlace = std::memcmp(seen.Node.Pivot, n0.Pivot, sizeof n0.Pivot) == 0 &&
			std::memcmp(&seen.Node.ClipRadius, &n0.ClipRadius, sizeof(float)) == 0;
		const bool sameCode = to - from == seen.Code.size() && to <= image.size() &&
			std::memcmp(image.data() + from, seen.Code.data(), seen.Code.size() * sizeof(float)) == 0;
		if (!samePlace || !sameCode || seen.Node.StackSize > n0.StackSize || seen.Node.StackSize < 1)
		{
			SetError(!samePlace ? "root pivot or clip radius differs from node 0" : !sameCode ?
				"root program differs from node 0's distance program" : "root program stack size out of range");
			return TG_ERR_INVALID;
		}
		if (code_quads) *code_quads = (int64_t)(seen.Code.size() / 4);
		if (stack_size) *stack_size = seen.Node.StackSize;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_debug_deferred_surfaces_check(void* tree)
	{
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		CompiledTree whole, later;
		std::string err;
		if (!CompileTree(Borrow(tree), whole, err)) { SetError(err); return TG_ERR_UNBOUNDED; }
		if (!CompileTree(Borrow(tree), later, err, OctreeKind::Export, nullptr, true)) { SetError(err); return TG_ERR_UNBOUNDED; }
		if (!later.Pending) { SetError("the deferred compile left nothing pending"); return TG_ERR_INVALID; }
		std::vector<float> a(whole.CodeFloats), b(later.CodeFloats);
		whole.CopyCode(a.data());
		later.CopyCode(b.data());
		if (!FinishSurfaces(later, b.data(), err)) { SetError(err); return TG_ERR_INVALID; }
		const bool same = a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(float)) == 0 &&
			whole.Nodes.size() == later.Nodes.size() &&
			std::memcmp(whole.Nodes.data(), later.Nodes.data(), whole.Nodes.size() * sizeof(OctNode)) == 0 &&
			std::memcmp(&whole.Header, &later.Header, sizeof(ProgramHeader)) == 0;
		if (!same) { SetError("the image with deferred surface programs differs from the whole compile's"); return TG_ERR_INVALID; }
		return TG_OK;
	}

	TANGERINE_API tg_status tg_debug_sodapop_plan(void* tree, float density, float* grid, int64_t* boxes, int64_t box_capacity,
		int64_t* leaves)
	{
		if (!tree || !grid) { SetError("null argument"); return TG_ERR_INVALID; }
		CompiledTree t;
		std::string err;
		if (!CompileTree(Borrow(tree), t, err, OctreeKind::Meshing)) { SetError(err); return TG_ERR_UNBOUNDED; }
		SodapopGrid g;
		std::vector<int64_t> b;
		if (!SodapopPlan(t, density, g, b, err)) { SetError(err); return TG_ERR_UNSUPPORTED; }
		grid[0] = g.G[0]; grid[1] = g.G[1]; grid[2] = g.G[2];
		grid[3] = g.D[0]; grid[4] = g.D[1]; grid[5] = g.D[2];
		grid[6] = (float)g.SX; grid[7] = (float)g.SY; grid[8] = (float)g.SZ;
		grid[9] = (float)g.Limit; grid[10] = (float)g.LZ;
		for (int64_t i = 0; i < (int64_t)b.size() && i < box_capacity * 6 && boxes; ++i) boxes[i] = b[(size_t)i];
		if (leaves) *leaves = (int64_t)(b.size() / 6);
		return TG_OK;
	}
}

namespace
{
	int64_t DumpOctree(const Octree& o, float* cells, int32_t* children, int64_t cell_capacity, uint32_t* words,
		int64_t word_capacity, int64_t* word_count)
	{
		int64_t w = 0;
		for (size_t i = 0; i < o.Cells.size(); ++i)
		{
			const Octree::Cell& c = o.Cells[i];
			std::vector<uint32_t> prog;
			if (c.Evaluator) prog = CompileReferenceWords(*c.Evaluator);
			if ((int64_t)i < cell_capacity && cells)
			{
				float* n = cells + i * 14;
				n[0] = c.Pivot.x; n[1] = c.Pivot.y; n[2] = c.Pivot.z;
				n[3] = c.Bounds.Min.x; n[4] = c.Bounds.Min.y; n[5] = c.Bounds.Min.z;
				n[6] = c.Bounds.Max.x; n[7] = c.Bounds.Max.y; n[8] = c.Bounds.Max.z;
				n[9] = c.Terminus ? 1.0f : 0.0f;
				n[10] = c.Evaluator ? 1.0f : 0.0f;
				n[11] = (float)w;
				n[12] = (float)prog.size();
				n[13] = c.Evaluator ? (float)c.Evaluator->StackSize : 0.0f;
			}
			if ((int64_t)i < cell_capacity && children)
			{
				for (int k = 0; k < 8; ++k) children[i * 8 + k] = c.Children[k];
			}
			for (uint32_t v : prog)
			{
				if (words && w < word_capacity) words[w] = v;
				++w;
			}
		}
		if (word_count) *word_count = w;
		return (int64_t)o.Cells.size();
	}
}

extern "C"
{

	TANGERINE_API tg_status tg_export_grid(const float lo[3], const float hi[3], float step, tg_grid* out)
	{
		if (!lo || !hi || !out || !(step > 0.0f)) { SetError("invalid export bounds"); return TG_ERR_INVALID; }
		ExportLattice(Vec3(lo[0], lo[1], lo[2]), Vec3(hi[0], hi[1], hi[2]), Vec3(step), *out);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_export_grid_axes(const float lo[3], const float hi[3], const float step[3], tg_grid* out)
	{
		if (!lo || !hi || !out || !step || !(step[0] > 0.0f) || !(step[1] > 0.0f) || !(step[2] > 0.0f))
		{
			SetError("invalid export bounds");
			return TG_ERR_INVALID;
		}
		ExportLattice(Vec3(lo[0], lo[1], lo[2]), Vec3(hi[0], hi[1], hi[2]), Vec3(step[0], step[1], step[2]), *out);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_eval_grid(tg_program* p, const tg_grid* g, float* out, int out_is_device, void* stream)
	{
		if (!p || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		GridSpec gs;
		if (!ToGridSpec(g, gs)) return TG_ERR_INVALID;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t s = StreamOf(stream);
		const size_t bytes = (size_t)g->nx * g->ny * g->nz * sizeof(float);
		float* dst = out;
		if (!out_is_device)
		{
			cudaError_t e = eng.Lattice().Reserve(bytes);
			if (e != cudaSuccess) return CudaFail(e, "allocating the lattice");
			dst = eng.Lattice().As<float>();
		}
		cudaError_t e = eng.EvalGrid(*p, gs, dst, s);
		if (e == cudaSuccess && !out_is_device) e = cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		if (e != cudaSuccess) return CudaFail(e, "evaluating the lattice");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_eval_points(tg_program* p, const float* points, int64_t n, float* out, void* stream)
	{
		if (!p || (n > 0 && (!points || !out))) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = eng.EvalPoints(*p, points, n, out, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "evaluating points");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_export_mesh_device(tg_program* p, const tg_grid* g, uint32_t flags, tg_device_mesh* out, void* stream)
	{
		if (!p || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		GridSpec gs;
		if (!ToGridSpec(g, gs)) return TG_ERR_INVALID;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		DeviceMesh dm;
		if (((flags >> 8) & 0xFFu) > 32) { SetError("brick size must be 1..32 cells"); return TG_ERR_INVALID; }
		cudaError_t e = eng.Export(*p, gs, OptionsOf(flags), dm, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "exporting the mesh");
		out->vertex_count = dm.VertexCount;
		out->face_count = dm.FaceCount;
		out->vertices = dm.Vertices;
		out->normals = dm.Normals;
		out->colors = dm.Colors;
		out->faces = dm.Faces;
		out->cubes = dm.Cubes;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_export_mesh(tg_program* p, const tg_grid* g, uint32_t flags, tg_mesh* out, void* stream)
	{
		if (!p || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		GridSpec gs;
		if (!ToGridSpec(g, gs)) return TG_ERR_INVALID;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t s = StreamOf(stream);
		DeviceMesh dm;
		if (((flags >> 8) & 0xFFu) > 32) { SetError("brick size must be 1..32 cells"); return TG_ERR_INVALID; }
		ExportOptions opt = OptionsOf(flags);
		HostMeshOut host;
		opt.Host = &host;
		const cudaError_t e = eng.Export(*p, gs, opt, dm, s);
		return TakeHostMesh(e, host, out, "exporting the mesh");
	}

	TANGERINE_API void tg_mesh_free(tg_mesh* m)
	{
		if (!m) return;
		void* blocks[5] = { m->vertices, m->normals, m->colors, m->faces, m->cubes };
		for (void* b : blocks)
		{
			if (!HostPool::Get().Give(b)) std::free(b);
		}
		std::memset(m, 0, sizeof *m);
	}

	TANGERINE_API tg_status tg_export_tree(void* tree, const float lo[3], const float hi[3], float step, tg_mesh* out, void* stream)
	{
		if (!out || !lo || !hi) { SetError("null argument"); return TG_ERR_INVALID; }
		tg_grid g;
		tg_status st = tg_export_grid(lo, hi, step, &g);
		if (st != TG_OK) return st;
		GridSpec gs;
		if (!ToGridSpec(&g, gs)) return TG_ERR_INVALID;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		ExportTiming& tm = LastTiming();
		auto clock = []() { return std::chrono::steady_clock::now(); };
		auto secs = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b)
		{
			return std::chrono::duration<double>(b - a).count();
		};
		const auto t0 = clock();
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		std::unique_ptr<tg_program> prog(new (std::nothrow) tg_program());
		if (!prog) { SetError("out of host memory"); return TG_ERR_MEMORY; }
		std::string err;
		const cudaStream_t s = StreamOf(stream);
		ExportOptions opt = OptionsOf(TG_MESH_ATTRIBUTES);
		// The exact brick test runs on the root cell's program, which exists right after
		// the root clip: the GPU classifies the bricks while the host builds the octree
		// below the root and emits its programs.
		cudaError_t pre = cudaErrorNotReady;
		const RootHook onRoot = [&](const RootProgram& r) { pre = eng.PreClassify(r, gs, opt.BrickSize, s); };
		// The surface programs (read by the normal and colour pass only) are left out of the
		// compile: the export emits them into the staged image while it waits for its
		// first read-back, and copies the code to the device again before that pass.
		if (!CompileTree(Borrow(tree), prog->Host, err, OctreeKind::Export, opt.Dense ? nullptr : &onRoot, true))
		{
			SetError(err);
			return TG_ERR_UNBOUNDED;
		}
		// Without the early test (an allocation failed, or none ran) the export classifies
		// as usual.
		if (pre != cudaSuccess && pre != cudaErrorNotReady) cudaGetLastError();
		opt.PreClassified = pre == cudaSuccess;
		cudaError_t ue = eng.UploadScratch(*prog, s);
		if (ue != cudaSuccess) return CudaFail(ue, "uploading the program");
		const auto t1 = clock();
		std::string surfaceError;
		opt.WhileWaiting = [&]() -> cudaError_t
		{
			return FinishSurfaces(prog->Host, eng.StagedCode(*prog), surfaceError) ? cudaSuccess : cudaErrorInvalidValue;
		};
		opt.RestageCode = true;
		DeviceMesh dm;
		HostMeshOut host;
		opt.Host = &host;
		const cudaError_t e = eng.Export(*prog, gs, opt, dm, s);
		const auto t2 = clock();
		if (!surfaceError.empty())
		{
			FreeHostMesh(host);
			std::memset(out, 0, sizeof *out);
			SetError(surfaceError);
			return TG_ERR_INVALID;
		}
		st = TakeHostMesh(e, host, out, "exporting the mesh");
		const auto t3 = clock();
		tm.CompileSeconds = prog->Host.BuildSeconds;
		tm.UploadSeconds = secs(t0, t1) - prog->Host.BuildSeconds;
		tm.GpuSeconds = secs(t1, t2);
		tm.CopySeconds = secs(t2, t3);
		return st;
	}

	TANGERINE_API tg_status tg_export_point_cloud(tg_program* p, const float lo[3], const float hi[3], const float step[3],
		int refine_iterations, uint32_t flags, tg_mesh* out, void* stream)
	{
		if (!p || !lo || !hi || !step || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		std::memset(out, 0, sizeof *out);
		if (refine_iterations < 0) { SetError("negative refinement count"); return TG_ERR_INVALID; }
		CloudSpec cs;
		std::string err;
		if (!CloudPlan(lo, hi, step, cs, err)) { SetError(err); return TG_ERR_UNSUPPORTED; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t s = StreamOf(stream);
		DeviceMesh dm;
		cudaError_t e = eng.PointCloud(*p, cs, refine_iterations, (flags & TG_MESH_ATTRIBUTES) != 0, dm, s);
		if (e != cudaSuccess) return CudaFail(e, "exporting the point cloud");
		return CopyMeshToHost(dm, out, s);
	}

	TANGERINE_API tg_status tg_export_voxels(tg_program* p, float grid_size, int color_index, tg_voxels* out, void* stream)
	{
		if (!p || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		std::memset(out, 0, sizeof *out);
		VoxSpec vs;
		std::string err;
		if (!VoxPlan(p->Host.Bounds, grid_size, vs, err)) { SetError(err); return TG_ERR_UNSUPPORTED; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		std::vector<uint32_t> cells;
		cudaError_t e = eng.Voxels(*p, vs, cells, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "voxelising the tree");
		out->voxels = (int32_t*)std::malloc(sizeof(int32_t) * 4 * (cells.empty() ? 1 : cells.size()));
		if (!out->voxels) { SetError("out of host memory for the voxels"); return TG_ERR_MEMORY; }
		// int z = i / Slice, y = (i % Slice) / Size.x, x = i % Size.x; abs(ColorIndex) % 255 + 1
		const int32_t slice = vs.SX * vs.SY;
		const int32_t color = std::abs(color_index) % 255 + 1;
		for (size_t v = 0; v < cells.size(); ++v)
		{
			const int32_t i = (int32_t)cells[v];
			out->voxels[v * 4 + 0] = i % vs.SX;
			out->voxels[v * 4 + 1] = (i % slice) / vs.SX;
			out->voxels[v * 4 + 2] = i / slice;
			out->voxels[v * 4 + 3] = color;
		}
		out->count = cells.size();
		out->size[0] = vs.SX; out->size[1] = vs.SY; out->size[2] = vs.SZ;
		out->radius = vs.Radius;
		return TG_OK;
	}

	TANGERINE_API void tg_voxels_free(tg_voxels* v)
	{
		if (!v) return;
		std::free(v->voxels);
		std::memset(v, 0, sizeof *v);
	}

	TANGERINE_API tg_status tg_write_vox(const tg_voxels* v, const char* path)
	{
		if (!v || !path || (v->count && !v->voxels)) { SetError("null argument"); return TG_ERR_INVALID; }
		if (!WriteVoxFile(path, v->size, v->voxels, (size_t)v->count)) { WriteFileError(path); return TG_ERR_IO; }
		return TG_OK;
	}

	TANGERINE_API void ExportMagicaVoxel(void* h, float grid_size, int color_index, const char* path)
	{
		if (!h || !path) { SetError("invalid export arguments"); return; }
		tg_program* prog = nullptr;
		if (tg_compile(h, &prog) != TG_OK) return;
		tg_voxels v;
		if (tg_export_voxels(prog, grid_size, color_index, &v, nullptr) == TG_OK)
		{
			tg_write_vox(&v, path);
			tg_voxels_free(&v);
		}
		tg_program_free(prog);
	}

	TANGERINE_API tg_status MeshExport(void* h, const char* path, const float lo[3], const float hi[3], const float step[3],
		int refine_iterations, int format, bool point_cloud, float scale)
	{
		if (!h || !path || !lo || !hi || !step) { SetError("invalid export arguments"); return TG_ERR_INVALID; }
		if (format != 0 && format != 1)
		{
			SetError("MeshExport writes STL (0) or PLY (1); MagicaVoxel files come from ExportMagicaVoxel");
			return TG_ERR_UNSUPPORTED;
		}
		if (point_cloud && format != 1)
		{
			SetError("the point-cloud export writes PLY only");
			return TG_ERR_UNSUPPORTED;
		}
		if (!(step[0] > 0.0f) || !(step[1] > 0.0f) || !(step[2] > 0.0f))
		{
			SetError("the export step must be positive on every axis");
			return TG_ERR_INVALID;
		}
		ExportJob& j = Job();
		{
			std::lock_guard<std::mutex> l(j.M);
			if (j.Running) { SetError("an export is already running (tg_export_result waits for it)"); return TG_ERR_BUSY; }
			// MeshExport (export.cpp:566-580): active, every progress word reset, stage 1.
			j.Running = true;
			j.Result = TG_OK;
			j.Error.clear();
			j.Active.store(true);
			j.Stage.store(0);
			j.Generation.store(0.0f);
			j.Refinement.store(0.0f);
			j.Secondary.store(0.0f);
			j.Write.store(0.0f);
			j.Stage.store(1);
		}
		ExportArgs args;
		args.Tree = Borrow(h);              // the job holds its own reference to the tree
		args.Path = path;
		for (int a = 0; a < 3; ++a) { args.Lo[a] = lo[a]; args.Hi[a] = hi[a]; args.Step[a] = step[a]; }
		args.Refine = refine_iterations;
		args.Format = format;
		args.PointCloud = point_cloud;
		args.Scale = scale;
		try
		{
			std::thread(RunExportJob, std::move(args)).detach();
		}
		catch (...)
		{
			{
				std::lock_guard<std::mutex> l(j.M);
				j.Running = false;
				j.Stage.store(0);
			}
			j.CV.notify_all();
			SetError("cannot start the export thread");
			return TG_ERR_MEMORY;
		}
		return TG_OK;
	}

	TANGERINE_API ExportProgress GetExportProgress(void)
	{
		ExportJob& j = Job();
		ExportProgress p;
		p.Stage = j.Stage.load();
		p.Generation = j.Generation.load();
		p.Refinement = j.Refinement.load();
		p.Secondary = j.Secondary.load();
		p.Write = j.Write.load();
		return p;
	}

	TANGERINE_API void CancelExport(bool halt)
	{
		ExportJob& j = Job();
		{
			std::lock_guard<std::mutex> l(j.M);
			if (halt) j.Active.store(false);
			else j.Stage.fetch_add(1);
		}
		j.CV.notify_all();
	}

	TANGERINE_API tg_status tg_export_result(int wait)
	{
		ExportJob& j = Job();
		std::unique_lock<std::mutex> l(j.M);
		if (wait) j.CV.wait(l, [&]() { return !j.Running; });
		else if (j.Running) { SetError("the export is still running"); return TG_ERR_BUSY; }
		if (j.Result != TG_OK) SetError(j.Error);
		return j.Result;
	}

	// Test hook: the next asynchronous export waits at the start of `stage` (1: before the
	// compile, 3: before the file write) until this is called with another stage or the export
	// is halted; the wait gives up after 30 s.  0 disarms.
	TANGERINE_API void tg_debug_export_pause(int stage)
	{
		ExportJob& j = Job();
		{
			std::lock_guard<std::mutex> l(j.M);
			j.PauseAt = stage;
		}
		j.CV.notify_all();
	}

	// 1 once the export waits at the armed stage (within timeout_ms), else 0.
	TANGERINE_API int tg_debug_export_paused(int timeout_ms)
	{
		ExportJob& j = Job();
		std::unique_lock<std::mutex> l(j.M);
		return j.CV.wait_for(l, std::chrono::milliseconds(timeout_ms), [&]() { return j.Paused; }) ? 1 : 0;
	}

	TANGERINE_API tg_status tg_sodapop_mesh(void* tree, float density, tg_drawable* out, void* stream)
	{
		if (!out) { SetError("null argument"); return TG_ERR_INVALID; }
		std::memset(out, 0, sizeof *out);
		if (!tree) { SetError("null tree handle"); return TG_ERR_INVALID; }
		const auto t0 = std::chrono::steady_clock::now();
		std::unique_ptr<tg_program> prog(new (std::nothrow) tg_program());
		if (!prog) { SetError("out of host memory"); return TG_ERR_MEMORY; }
		std::string err;
		if (!CompileTree(Borrow(tree), prog->Host, err, OctreeKind::Meshing))
		{
			SetError(err);
			return TG_ERR_UNBOUNDED;
		}
		SodapopGrid g;
		std::vector<int64_t> boxes;
		if (!SodapopPlan(prog->Host, density, g, boxes, err))
		{
			SetError(err);
			return TG_ERR_UNSUPPORTED;
		}
		const auto t1 = std::chrono::steady_clock::now();
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t s = StreamOf(stream);
		cudaError_t e = eng.UploadScratch(*prog, s);
		if (e != cudaSuccess) return CudaFail(e, "uploading the program");
		SodapopMesh m;
		e = eng.Sodapop(*prog, g, boxes, m, s);
		if (e != cudaSuccess) return CudaFail(e, "running the meshing job");
		auto take = [](size_t bytes) -> void*
		{
			void* p = HostPool::Get().Take(bytes);
			return p ? p : std::malloc(bytes);
		};
		const size_t v = m.VertexCount ? m.VertexCount : 1, f = m.FaceCount ? m.FaceCount : 1;
		out->positions = (float*)take(v * 12);
		out->normals = (float*)take(v * 12);
		out->colors = (float*)take(v * 16);
		out->faces = (uint32_t*)take(f * 12);
		out->cells = (uint32_t*)take(v * 4);
		if (!out->positions || !out->normals || !out->colors || !out->faces || !out->cells)
		{
			tg_drawable_free(out);
			SetError("out of host memory for the drawable");
			return TG_ERR_MEMORY;
		}
		out->vertex_count = m.VertexCount;
		out->face_count = m.FaceCount;
		if (m.VertexCount)
		{
			e = cudaMemcpyAsync(out->positions, m.Positions, m.VertexCount * 12, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaMemcpyAsync(out->normals, m.Normals, m.VertexCount * 12, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaMemcpyAsync(out->colors, m.Colors, m.VertexCount * 16, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaMemcpyAsync(out->cells, m.Cells, m.VertexCount * 4, cudaMemcpyDeviceToHost, s);
		}
		if (e == cudaSuccess && m.FaceCount) e = cudaMemcpyAsync(out->faces, m.Faces, m.FaceCount * 12, cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		if (e != cudaSuccess)
		{
			tg_drawable_free(out);
			return CudaFail(e, "copying the drawable to the host");
		}
		for (int a = 0; a < 3; ++a)
		{
			out->grid_origin[a] = g.G[a];
			out->grid_step[a] = g.D[a];
		}
		out->grid_cells[0] = g.SX; out->grid_cells[1] = g.SY; out->grid_cells[2] = g.SZ;
		const auto t2 = std::chrono::steady_clock::now();
		out->compile_seconds = std::chrono::duration<double>(t1 - t0).count();
		out->gpu_seconds = std::chrono::duration<double>(t2 - t1).count();
		return TG_OK;
	}

	TANGERINE_API void tg_drawable_free(tg_drawable* d)
	{
		if (!d) return;
		void* blocks[5] = { d->positions, d->normals, d->colors, d->faces, d->cells };
		for (void* b : blocks)
		{
			if (!HostPool::Get().Give(b)) std::free(b);
		}
		std::memset(d, 0, sizeof *d);
	}

	TANGERINE_API tg_status tg_ray_query(tg_program* p, int mode, const float frame[8], const float* origins, const float* dirs, int64_t n,
		int iterations, float epsilon, uint8_t* hit, float* travel, float* position, void* stream)
	{
		if (!p || (n > 0 && (!origins || !dirs || !hit || !travel || !position))) { SetError("null argument"); return TG_ERR_INVALID; }
		if (mode < 0 || mode > 2 || (mode == 2 && !frame)) { SetError("ray mode is 0, 1 or 2 (2 needs a frame)"); return TG_ERR_INVALID; }
		if (iterations < 0) { SetError("negative iteration count"); return TG_ERR_INVALID; }
		RayFrame f{};
		f.Mode = mode;
		f.Rotation[0] = 1.0f;
		f.Scale = 1.0f;
		if (mode == 2)
		{
			for (int k = 0; k < 4; ++k) f.Rotation[k] = frame[k];
			for (int k = 0; k < 3; ++k) f.Translation[k] = frame[4 + k];
			f.Scale = frame[7];
			// SDFModel::RayMarch passes 1000 iterations and RayMarch's default epsilon.
			iterations = 1000;
			epsilon = 0.001f;
		}
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = eng.RayMarch(*p, origins, dirs, n, iterations, epsilon, hit, travel, position, StreamOf(stream), &f);
		if (e != cudaSuccess) return CudaFail(e, "casting rays");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_eval_tree_points(tg_program* p, const float* points, int64_t n, float* out, void* stream)
	{
		if (!p || (n > 0 && (!points || !out))) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = eng.PointQuery(*p, points, n, false, out, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "evaluating the tree");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_gradient_tree_points(tg_program* p, const float* points, int64_t n, float* out, void* stream)
	{
		if (!p || (n > 0 && (!points || !out))) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = eng.PointQuery(*p, points, n, true, out, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "taking gradients");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_ray_march(tg_program* p, const float* origins, const float* dirs, int64_t n, int iterations, float epsilon,
		uint8_t* hit, float* travel, float* position, void* stream)
	{
		if (!p || (n > 0 && (!origins || !dirs || !hit || !travel || !position))) { SetError("null argument"); return TG_ERR_INVALID; }
		if (iterations < 0) { SetError("negative iteration count"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = eng.RayMarch(*p, origins, dirs, n, iterations, epsilon, hit, travel, position, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "ray marching");
		return TG_OK;
	}

	namespace
	{
		tg_status RenderWith(tg_program* p, tg_surrogate* field, const tg_camera* cameras, int count, int width, int height, int max_steps,
			float epsilon, uint32_t flags, float* depth, float* normals, uint8_t* colors, int out_is_device, void* stream)
		{
			if (!p || !cameras || !depth || !normals) { SetError("null argument"); return TG_ERR_INVALID; }
			if (count < 0 || width <= 0 || height <= 0 || max_steps < 0) { SetError("invalid image size or step count"); return TG_ERR_INVALID; }
			std::vector<CameraBasis> basis((size_t)count);
			for (int c = 0; c < count; ++c)
			{
				const tg_camera& cam = cameras[c];
				const Vec3 pos(cam.position[0], cam.position[1], cam.position[2]);
				const Vec3 fwd = Normalize(Vec3(cam.target[0], cam.target[1], cam.target[2]) - pos);
				const Vec3 right = Normalize(Cross(fwd, Vec3(cam.up[0], cam.up[1], cam.up[2])));
				const Vec3 up = Cross(right, fwd);
				CameraBasis& b = basis[(size_t)c];
				b.Position[0] = pos.x; b.Position[1] = pos.y; b.Position[2] = pos.z;
				b.Forward[0] = fwd.x; b.Forward[1] = fwd.y; b.Forward[2] = fwd.z;
				b.Right[0] = right.x; b.Right[1] = right.y; b.Right[2] = right.z;
				b.Up[0] = up.x; b.Up[1] = up.y; b.Up[2] = up.z;
				b.TanHalfFov = cam.tan_half_fov;
				b.Aspect = (float)width / (float)height;
			}
			Engine& eng = Engine::Get();
			std::lock_guard<std::mutex> lock(eng.Mutex);
			cudaError_t e = eng.Render(*p, basis.data(), count, width, height, max_steps, epsilon, (flags & TG_RENDER_EXACT) != 0, depth,
				normals, p->Host.Header.HasPaint ? colors : nullptr, out_is_device != 0, StreamOf(stream), field);
			if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the network renderer"); return TG_ERR_CUDA; }
			if (e != cudaSuccess) return CudaFail(e, "rendering");
			if (colors && !p->Host.Header.HasPaint && !out_is_device)
				std::memset(colors, 255, (size_t)width * height * count * 3);
			return TG_OK;
		}
	}

	TANGERINE_API tg_status tg_render(tg_program* p, const tg_camera* cameras, int count, int width, int height, int max_steps,
		float epsilon, uint32_t flags, float* depth, float* normals, uint8_t* colors, int out_is_device, void* stream)
	{
		return RenderWith(p, nullptr, cameras, count, width, height, max_steps, epsilon, flags, depth, normals, colors, out_is_device,
			stream);
	}

	TANGERINE_API tg_status tg_render_surrogate(tg_program* p, tg_surrogate* net, const tg_camera* cameras, int count, int width,
		int height, int max_steps, float epsilon, float* depth, float* normals, uint8_t* colors, int out_is_device, void* stream)
	{
		if (!net) { SetError("null surrogate"); return TG_ERR_INVALID; }
		return RenderWith(p, net, cameras, count, width, height, max_steps, epsilon, 0, depth, normals, colors, out_is_device, stream);
	}

	TANGERINE_API tg_status tg_last_render_steps(uint64_t* network_steps, uint64_t* exact_steps)
	{
		Engine& eng = Engine::Get();
		if (network_steps) *network_steps = eng.LastNetworkSteps;
		if (exact_steps) *exact_steps = eng.LastExactSteps;
		return TG_OK;
	}

	// WritePLY (export.cpp:198-280): header, then x y z nx ny nz [r g b] per vertex, then
	// "3 i j k" per face, little endian.  Positions are multiplied by `scale`.
	TANGERINE_API tg_status tg_write_ply(const tg_mesh* m, const char* path, float scale)
	{
		if (!m || !path) { SetError("null argument"); return TG_ERR_INVALID; }
		FILE* f = std::fopen(path, "wb");
		if (!f) { WriteFileError(path); return TG_ERR_IO; }
		const bool color = m->colors != nullptr;
		std::string header = "ply\nformat binary_little_endian 1.0\ncomment Created by Tangerine\n";
		header += "element vertex " + std::to_string(m->vertex_count) + "\n";
		header += "property float x\nproperty float y\nproperty float z\n";
		header += "property float nx\nproperty float ny\nproperty float nz\n";
		if (color) header += "property uchar red\nproperty uchar green\nproperty uchar blue\n";
		if (m->face_count > 0)
		{
			header += "element face " + std::to_string(m->face_count) + "\n";
			header += "property list uchar uint vertex_indices\n";
		}
		header += "end_header\n";
		bool ok = std::fwrite(header.data(), 1, header.size(), f) == header.size();
		const size_t stride = color ? 27 : 24;
		std::vector<uint8_t> buf(stride * (size_t)(m->vertex_count < 65536 ? m->vertex_count : 65536) + 16);
		for (uint64_t v0 = 0; ok && v0 < m->vertex_count; v0 += 65536)
		{
			const uint64_t n = (m->vertex_count - v0) < 65536 ? (m->vertex_count - v0) : 65536;
			uint8_t* o = buf.data();
			for (uint64_t v = v0; v < v0 + n; ++v)
			{
				const float pos[3] = { m->vertices[v * 3] * scale, m->vertices[v * 3 + 1] * scale, m->vertices[v * 3 + 2] * scale };
				std::memcpy(o, pos, 12);
				std::memcpy(o + 12, m->normals + v * 3, 12);
				if (color) std::memcpy(o + 24, m->colors + v * 3, 3);
				o += stride;
			}
			ok = std::fwrite(buf.data(), 1, (size_t)(o - buf.data()), f) == (size_t)(o - buf.data());
		}
		std::vector<uint8_t> fb(13 * 65536);
		for (uint64_t t0 = 0; ok && t0 < m->face_count; t0 += 65536)
		{
			const uint64_t n = (m->face_count - t0) < 65536 ? (m->face_count - t0) : 65536;
			uint8_t* o = fb.data();
			for (uint64_t t = t0; t < t0 + n; ++t)
			{
				*o = 3;
				std::memcpy(o + 1, m->faces + t * 3, 12);
				o += 13;
			}
			ok = std::fwrite(fb.data(), 1, (size_t)(o - fb.data()), f) == (size_t)(o - fb.data());
		}
		ok = (std::fclose(f) == 0) && ok;
		if (!ok) { WriteFileError(path); return TG_ERR_IO; }
		return TG_OK;
	}

	// WriteSTL(Octree, ...) (export.cpp:111-179): 80-byte header, count, then per triangle
	// the gradient at its centroid, its three corners (times `scale`) and a zero word.
	TANGERINE_API tg_status tg_write_stl(tg_program* p, const tg_mesh* m, const char* path, float scale, void* stream)
	{
		if (!p || !m || !path) { SetError("null argument"); return TG_ERR_INVALID; }
		std::vector<float> normals((size_t)m->face_count * 3);
		{
			Engine& eng = Engine::Get();
			std::lock_guard<std::mutex> lock(eng.Mutex);
			cudaError_t e = eng.FaceNormals(*p, m->vertices, m->vertex_count, m->faces, m->face_count, normals.data(), StreamOf(stream));
			if (e != cudaSuccess) return CudaFail(e, "computing face normals");
		}
		FILE* f = std::fopen(path, "wb");
		if (!f) { WriteFileError(path); return TG_ERR_IO; }
		char header[80];
		std::memset(header, 0, sizeof header);
		const char* title = "STL generated by TangerineCSG";
		std::memcpy(header, title, std::strlen(title));
		bool ok = std::fwrite(header, 1, 80, f) == 80;
		const uint32_t count = (uint32_t)m->face_count;
		ok = ok && std::fwrite(&count, 4, 1, f) == 1;
		std::vector<uint8_t> rec(50);
		for (uint64_t t = 0; ok && t < m->face_count; ++t)
		{
			std::memcpy(rec.data(), normals.data() + t * 3, 12);
			for (int c = 0; c < 3; ++c)
			{
				const uint32_t v = m->faces[t * 3 + c];
				const float pos[3] = { m->vertices[(size_t)v * 3] * scale, m->vertices[(size_t)v * 3 + 1] * scale, m->vertices[(size_t)v * 3 + 2] * scale };
				std::memcpy(rec.data() + 12 + 12 * c, pos, 12);
			}
			rec[48] = 0; rec[49] = 0;
			ok = std::fwrite(rec.data(), 1, 50, f) == 50;
		}
		ok = (std::fclose(f) == 0) && ok;
		if (!ok) { WriteFileError(path); return TG_ERR_IO; }
		return TG_OK;
	}

	TANGERINE_API tg_status tg_write_drawables(const tg_drawable* drawables, const float* frames, int count, const char* path,
		int format, float scale)
	{
		if ((count > 0 && !drawables) || !path || count < 0) { SetError("null argument"); return TG_ERR_INVALID; }
		if (format != 0 && format != 1) { SetError("format is 0 (STL) or 1 (PLY)"); return TG_ERR_INVALID; }
		// The gather of MeshExport(Path, UseBaseColor, ...) (export.cpp:495-548): positions
		// through the model's LocalToWorld matrix times Scale, normals as they are, colour
		// bytes 0xFF * c, indices offset by the vertices before.
		uint64_t nv = 0, nf = 0;
		for (int d = 0; d < count; ++d) { nv += drawables[d].vertex_count; nf += drawables[d].face_count; }
		std::vector<float> V((size_t)nv * 3), N((size_t)nv * 3);
		std::vector<uint8_t> Cb((size_t)nv * 3);
		std::vector<uint32_t> F((size_t)nf * 3);
		uint64_t vo = 0, fo = 0;
		for (int d = 0; d < count; ++d)
		{
			const tg_drawable& dr = drawables[d];
			Transform t;
			if (frames)
			{
				const float* fr = frames + (size_t)d * 8;
				t.Rotation = Quat{ fr[0], fr[1], fr[2], fr[3] };
				t.Translation = Vec3(fr[4], fr[5], fr[6]);
				t.Scalation = fr[7];
			}
			const Mat4 M = t.ToMatrix();
			for (uint64_t i = 0; i < dr.vertex_count; ++i)
			{
				const float x = dr.positions[i * 3], y = dr.positions[i * 3 + 1], z = dr.positions[i * 3 + 2];
				// (M * vec4(p, 1)).xyz = (m0*x + m1*y) + (m2*z + m3*1), then * vec3(Scale)
				for (int r = 0; r < 3; ++r)
				{
					const float w = (M.at(0, r) * x + M.at(1, r) * y) + (M.at(2, r) * z + M.at(3, r) * 1.0f);
					V[(size_t)(vo + i) * 3 + r] = w * scale;
					N[(size_t)(vo + i) * 3 + r] = dr.normals[i * 3 + r];
					// float -> integer -> low byte, as the x86 conversion into a uint8_t vector does
					Cb[(size_t)(vo + i) * 3 + r] = (uint8_t)(int32_t)(255.0f * dr.colors[i * 4 + r]);
				}
			}
			for (uint64_t f = 0; f < dr.face_count * 3; ++f) F[(size_t)(fo * 3 + f)] = (uint32_t)(vo + dr.faces[f]);
			vo += dr.vertex_count;
			fo += dr.face_count;
		}
		if (format == 1)
		{
			tg_mesh m{};
			m.vertex_count = nv;
			m.face_count = nf;
			m.vertices = V.data();
			m.normals = N.data();
			m.colors = Cb.data();
			m.faces = F.data();
			return tg_write_ply(&m, path, 1.0f);
		}
		// WriteSTL(Path, Vertices, Normals, Triangles) (export.cpp:60-108): each facet's normal
		// is normalize(N[a] + N[b] + N[c]); no padding follows (84 + 50n is a multiple of 4
		// whenever the reference's 84 + 100n is).
		FILE* out = std::fopen(path, "wb");
		if (!out) { WriteFileError(path); return TG_ERR_IO; }
		char header[80];
		std::memset(header, 0, sizeof header);
		const char* title = "STL generated by TangerineCSG";
		std::memcpy(header, title, std::strlen(title));
		bool ok = std::fwrite(header, 1, 80, out) == 80;
		const uint32_t tris = (uint32_t)nf;
		ok = ok && std::fwrite(&tris, 4, 1, out) == 1;
		uint8_t rec[50];
		for (uint64_t t = 0; ok && t < nf; ++t)
		{
			const uint32_t a = F[t * 3], b = F[t * 3 + 1], c = F[t * 3 + 2];
			Vec3 n(N[(size_t)a * 3], N[(size_t)a * 3 + 1], N[(size_t)a * 3 + 2]);
			n = n + Vec3(N[(size_t)b * 3], N[(size_t)b * 3 + 1], N[(size_t)b * 3 + 2]);
			n = n + Vec3(N[(size_t)c * 3], N[(size_t)c * 3 + 1], N[(size_t)c * 3 + 2]);
			n = Normalize(n);
			const float nn[3] = { n.x, n.y, n.z };
			std::memcpy(rec, nn, 12);
			std::memcpy(rec + 12, &V[(size_t)a * 3], 12);
			std::memcpy(rec + 24, &V[(size_t)b * 3], 12);
			std::memcpy(rec + 36, &V[(size_t)c * 3], 12);
			rec[48] = 0; rec[49] = 0;
			ok = std::fwrite(rec, 1, 50, out) == 50;
		}
		ok = (std::fclose(out) == 0) && ok;
		if (!ok) { WriteFileError(path); return TG_ERR_IO; }
		return TG_OK;
	}

	// ExportCommon (export.cpp:595-607): the tree's bounds at a 1/GridSize step.
	static void ExportToFile(void* h, float grid_size, const char* path, bool ply)
	{
		if (!h || !path || !(grid_size > 0.0f)) { SetError("invalid export arguments"); return; }
		const AABB b = AsNode(h)->Bounds();
		const float step = (float)(1.0 / (double)grid_size);
		const float lo[3] = { b.Min.x, b.Min.y, b.Min.z }, hi[3] = { b.Max.x, b.Max.y, b.Max.z };
		tg_program* prog = nullptr;
		if (tg_compile(h, &prog) != TG_OK) return;
		tg_grid g;
		tg_mesh m;
		if (tg_export_grid(lo, hi, step, &g) == TG_OK && tg_export_mesh(prog, &g, TG_MESH_ATTRIBUTES, &m, nullptr) == TG_OK)
		{
			if (ply) tg_write_ply(&m, path, 1.0f);
			else tg_write_stl(prog, &m, path, 1.0f, nullptr);
			tg_mesh_free(&m);
		}
		tg_program_free(prog);
	}

	TANGERINE_API void ExportSTL(void* h, float grid_size, int, const char* path) { ExportToFile(h, grid_size, path, false); }
	TANGERINE_API void ExportPLY(void* h, float grid_size, int, const char* path) { ExportToFile(h, grid_size, path, true); }

	TANGERINE_API tg_status tg_last_export_stats(int64_t* bricks, int64_t* active_bricks)
	{
		if (bricks) *bricks = Engine::Get().LastBricks();
		if (active_bricks) *active_bricks = Engine::Get().LastActiveBricks();
		return TG_OK;
	}

	TANGERINE_API tg_status tg_last_export_timing(double* compile_s, double* upload_s, double* gpu_s, double* copy_s)
	{
		const ExportTiming& t = LastTiming();
		if (compile_s) *compile_s = t.CompileSeconds;
		if (upload_s) *upload_s = t.UploadSeconds;
		if (gpu_s) *gpu_s = t.GpuSeconds;
		if (copy_s) *copy_s = t.CopySeconds;
		return TG_OK;
	}

	TANGERINE_API void tg_profile_enable(int on) { Engine::Get().SetProfiling(on != 0); }
	TANGERINE_API int tg_profile_read(const char* name, double* ms, int64_t* launches)
	{
		double m = 0.0; int64_t n = 0;
		const bool found = Engine::Get().ReadProfile(name ? name : "", m, n);
		if (ms) *ms = m;
		if (launches) *launches = n;
		return found ? 1 : 0;
	}
	TANGERINE_API void tg_profile_reset(void) { Engine::Get().ResetProfile(); }

	TANGERINE_API tg_status tg_measure_fp32_peak(double* tflops, void* stream)
	{
		if (!tflops) { SetError("null argument"); return TG_ERR_INVALID; }
		std::lock_guard<std::mutex> lock(Engine::Get().Mutex);
		cudaError_t e = MeasureFp32Peak(tflops, StreamOf(stream));
		if (e != cudaSuccess) return CudaFail(e, "measuring FP32 throughput");
		return TG_OK;
	}

	// ---- many trees in one launch ---------------------------------------------------------

	TANGERINE_API tg_status tg_batch_create(tg_program* const* programs, const tg_grid* grids, int count, uint32_t flags, tg_batch** out)
	{
		if (!out || !programs || !grids || count <= 0) { SetError("null argument"); return TG_ERR_INVALID; }
		*out = nullptr;
		std::vector<const Program*> progs((size_t)count);
		std::vector<GridSpec> specs((size_t)count);
		for (int m = 0; m < count; ++m)
		{
			if (!programs[m]) { SetError("null program in the batch"); return TG_ERR_INVALID; }
			progs[m] = programs[m];
			if (!ToGridSpec(&grids[m], specs[m])) return TG_ERR_INVALID;
		}
		std::unique_ptr<tg_batch> b(new (std::nothrow) tg_batch(std::move(progs), std::move(specs), (flags & TG_MESH_ATTRIBUTES) != 0));
		if (!b) { SetError("out of host memory"); return TG_ERR_MEMORY; }
		*out = b.release();
		return TG_OK;
	}

	TANGERINE_API void tg_batch_free(tg_batch* b)
	{
		if (!b) return;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		delete b;
	}

	TANGERINE_API tg_status tg_batch_autotune(tg_batch* b, void* stream)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = b->Autotune(StreamOf(stream));
		return e == cudaSuccess ? TG_OK : CudaFail(e, "autotuning the batch");
	}

	TANGERINE_API tg_status tg_batch_set_tuning(tg_batch* b, const int* bricks, const int* lanes)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		const size_t n = b->Bricks.size();
		std::vector<int> bv = b->Bricks, lv = b->Lanes;
		for (size_t m = 0; m < n; ++m)
		{
			if (bricks && (bricks[m] < 1 || bricks[m] > 32)) { SetError("brick edge must be 1..32 cells"); return TG_ERR_INVALID; }
			if (lanes && lanes[m] != 1 && lanes[m] != 2 && lanes[m] != 4) { SetError("lanes must be 1, 2 or 4"); return TG_ERR_INVALID; }
			if (bricks) bv[m] = bricks[m];
			if (lanes) lv[m] = lanes[m];
		}
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		b->SetTuning(bv, lv);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_set_surrogates(tg_batch* b, tg_surrogate* const* nets, int count, uint32_t flags)
	{
		if (!b || (count > 0 && !nets) || count < 0) { SetError("null argument"); return TG_ERR_INVALID; }
		std::vector<const FieldNet*> fields((size_t)count);
		for (int m = 0; m < count; ++m) fields[(size_t)m] = nets[m];
		b->SetFields(fields, (flags & TG_MESH_SURROGATE_ONLY) == 0);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_get_tuning(const tg_batch* b, int* bricks, int* lanes)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		for (size_t m = 0; m < b->Bricks.size(); ++m)
		{
			if (bricks) bricks[m] = b->Bricks[m];
			if (lanes) lanes[m] = b->Lanes[m];
		}
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_run(tg_batch* b, void* stream)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = b->Run(StreamOf(stream));
		if (e == cudaErrorLaunchTimeout) return TG_ERR_CUDA;
		if (e == cudaSuccess && b->LastStatus == 3) return TG_ERR_CANCELLED;
		return e == cudaSuccess ? TG_OK : CudaFail(e, "running the batch");
	}

	TANGERINE_API tg_status tg_batch_cancel(tg_batch* b, int cancel)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		if (!b->SetCancel(cancel != 0)) { SetError("cannot map the batch's cancel flag (wrong device current?)"); return TG_ERR_CUDA; }
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_debug_barrier(tg_batch* b, uint64_t limit_ns, int late_block, uint64_t late_ns)
	{
		if (!b) { SetError("null argument"); return TG_ERR_INVALID; }
		if (late_ns > 2000000000ull || limit_ns > 60000000000ull || (limit_ns && limit_ns < 1000000ull))
		{
			SetError("barrier limit must be 0 or 1 ms..60 s, the late start at most 2 s");
			return TG_ERR_INVALID;
		}
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		b->SetBarrierKnobs(limit_ns, late_block, late_ns);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_debug_wait_test(int which, uint64_t limit_ns)
	{
		if ((which != 0 && which != 1) || limit_ns > 1000000000ull)
		{
			SetError("wait test: which is 0 (staged program copy) or 1 (network image), the limit at most 1 s");
			return TG_ERR_INVALID;
		}
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaError_t e = which == 0 ? SetStageWaitTest(limit_ns) : SetSetupWaitTest(limit_ns);
		if (e != cudaSuccess) return CudaFail(e, "setting a wait test hook");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_reserve(tg_batch* b, uint64_t vertices, uint64_t faces)
	{
		if (!b || vertices >= (1ull << 32) || faces >= (1ull << 32)) { SetError("invalid argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		b->Reserve((uint32_t)vertices, (uint32_t)faces);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_get_info(const tg_batch* b, tg_batch_info* out)
	{
		if (!b || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		const BatchInfo& i = b->Info;
		out->models = i.Models;
		out->samples = i.Samples;
		out->bricks = i.Bricks;
		out->bricks_evaluated = i.BricksEvaluated;
		out->vertices = i.Vertices;
		out->faces = i.Faces;
		out->graph = i.Graph;
		out->blocks = i.Blocks;
		out->reruns = i.Reruns;
		out->autotune_seconds = i.AutotuneSeconds;
		out->device_bytes = i.DeviceBytes;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_mesh_device(tg_batch* b, int model, tg_device_mesh* out)
	{
		if (!b || !out || model < 0 || model >= (int)b->Bricks.size()) { SetError("invalid argument"); return TG_ERR_INVALID; }
		DeviceMesh dm;
		b->MeshOf(model, dm);
		out->vertex_count = dm.VertexCount;
		out->face_count = dm.FaceCount;
		out->vertices = dm.Vertices;
		out->normals = dm.Normals;
		out->colors = dm.Colors;
		out->faces = dm.Faces;
		out->cubes = dm.Cubes;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_batch_mesh(tg_batch* b, int model, tg_mesh* out, void* stream)
	{
		if (!b || !out || model < 0 || model >= (int)b->Bricks.size()) { SetError("invalid argument"); return TG_ERR_INVALID; }
		DeviceMesh dm;
		b->MeshOf(model, dm);
		return CopyMeshToHost(dm, out, StreamOf(stream));
	}

	// ---- learned distance bound ---------------------------------------------------------

	TANGERINE_API void tg_surrogate_default_options(tg_surrogate_options* o)
	{
		if (!o) return;
		const FieldOptions d;
		o->log2_table = d.Log2Table;
		o->base_resolution = d.BaseRes;
		o->max_resolution = d.MaxRes;
		for (int a = 0; a < 3; ++a) { o->domain_min[a] = d.Lo[a]; o->domain_max[a] = d.Hi[a]; }
		o->clamp = d.Clamp;
		o->samples = d.Samples;
		o->band = d.Band;
		o->batch = d.Batch;
		o->steps = d.Steps;
		o->learning_rate = d.Rate;
		o->validation = d.Validation;
		o->safety = d.Safety;
		o->seed = d.Seed;
	}

	TANGERINE_API tg_status tg_surrogate_create(const tg_surrogate_options* o, tg_surrogate** out)
	{
		if (!out) { SetError("null argument"); return TG_ERR_INVALID; }
		*out = nullptr;
		tg_surrogate_options def;
		tg_surrogate_default_options(&def);
		if (!o) o = &def;
		if (o->log2_table < 10 || o->log2_table > 24 || o->base_resolution < 1 || o->max_resolution < o->base_resolution ||
			o->max_resolution > (1 << 20) || !(o->clamp > 0.0f) || o->samples < 2 || o->batch < 1 || o->steps < 0 ||
			o->validation < 2 || !(o->safety >= 0.0f) || !(o->band > 0.0f))
		{
			SetError("invalid surrogate options");
			return TG_ERR_INVALID;
		}
		FieldOptions f;
		f.Log2Table = o->log2_table;
		f.BaseRes = o->base_resolution;
		f.MaxRes = o->max_resolution;
		for (int a = 0; a < 3; ++a)
		{
			if (!(o->domain_max[a] > o->domain_min[a])) { SetError("empty surrogate domain"); return TG_ERR_INVALID; }
			f.Lo[a] = o->domain_min[a];
			f.Hi[a] = o->domain_max[a];
		}
		f.Clamp = o->clamp;
		f.Samples = o->samples;
		f.Band = o->band;
		f.Batch = o->batch;
		f.Steps = o->steps;
		f.Rate = o->learning_rate;
		f.Validation = o->validation;
		f.Safety = o->safety;
		f.Seed = o->seed;
		std::unique_ptr<tg_surrogate> s(new (std::nothrow) tg_surrogate(f));
		if (!s) { SetError("out of host memory"); return TG_ERR_MEMORY; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = s->Init(eng.DefaultStream());
		if (e != cudaSuccess) return CudaFail(e, "allocating the surrogate");
		*out = s.release();
		return TG_OK;
	}

	TANGERINE_API void tg_surrogate_free(tg_surrogate* s) { delete s; }

	TANGERINE_API tg_status tg_surrogate_fit(tg_surrogate* s, tg_program* p, void* stream)
	{
		if (!s || !p) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = s->Fit(*p, StreamOf(stream));
		if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the surrogate kernels"); return TG_ERR_CUDA; }
		if (e != cudaSuccess) return CudaFail(e, "training the surrogate");
		return TG_OK;
	}

	TANGERINE_API tg_status tg_surrogate_get_info(const tg_surrogate* s, tg_surrogate_info* out)
	{
		if (!s || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		std::memset(out, 0, sizeof *out);
		out->max_error = s->Info.MaxError;
		out->p99_error = s->Info.P99Error;
		out->mean_error = s->Info.MeanError;
		out->margin = s->Info.Margin;
		out->final_loss = s->Info.FinalLoss;
		out->data_seconds = s->Info.DataSeconds;
		out->train_seconds = s->Info.TrainSeconds;
		out->samples = s->Info.Samples;
		out->steps = s->Info.Steps;
		for (int l = 0; l < kFieldLevels; ++l) out->resolutions[l] = s->Grid.Res[l];
		out->table_size = s->Grid.TableSize;
		out->dense_levels = s->Grid.DenseLevels;
		out->table_floats = s->TableFloats;
		out->mlp_floats = kFieldParams;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_surrogate_get_params(tg_surrogate* s, float* table, float* mlp)
	{
		if (!s) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = s->GetParams(table, mlp, eng.DefaultStream());
		return e == cudaSuccess ? TG_OK : CudaFail(e, "reading surrogate parameters");
	}

	TANGERINE_API tg_status tg_surrogate_set_params(tg_surrogate* s, const float* table, const float* mlp)
	{
		if (!s) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		cudaError_t e = s->SetParams(table, mlp, eng.DefaultStream());
		return e == cudaSuccess ? TG_OK : CudaFail(e, "writing surrogate parameters");
	}

	TANGERINE_API int64_t tg_surrogate_save(tg_surrogate* s, void* out, int64_t capacity)
	{
		if (!s || capacity < 0) { SetError("null argument"); return -1; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		std::vector<uint8_t> bytes;
		const cudaError_t e = s->Save(bytes, eng.DefaultStream());
		if (e != cudaSuccess) { CudaFail(e, "saving the surrogate"); return -1; }
		if (out)
		{
			if (capacity < (int64_t)bytes.size()) { SetError("checkpoint buffer too small"); return -1; }
			std::memcpy(out, bytes.data(), bytes.size());
		}
		return (int64_t)bytes.size();
	}

	TANGERINE_API tg_status tg_surrogate_load(tg_surrogate* s, const void* data, int64_t size)
	{
		if (!s || !data || size <= 0) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		std::string why;
		const cudaError_t e = s->Load(static_cast<const uint8_t*>(data), (size_t)size, why, eng.DefaultStream());
		if (e == cudaErrorInvalidValue && !why.empty()) { SetError(why); return TG_ERR_INVALID; }
		return e == cudaSuccess ? TG_OK : CudaFail(e, "loading the surrogate");
	}

	TANGERINE_API tg_status tg_surrogate_eval(tg_surrogate* s, const float* points, int64_t n, float* out, int io_is_device, void* stream)
	{
		if (!s || (n > 0 && (!points || !out)) || n < 0) { SetError("null argument"); return TG_ERR_INVALID; }
		if (n == 0) return TG_OK;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = StreamOf(stream);
		cudaError_t e = cudaSuccess;
		if (io_is_device) e = s->Eval(points, n, 3, out, st);
		else
		{
			DeviceBuffer dp, dout;
			e = dp.Reserve((size_t)n * 12);
			if (e == cudaSuccess) e = dout.Reserve((size_t)n * 4);
			if (e == cudaSuccess) e = cudaMemcpyAsync(dp.Ptr, points, (size_t)n * 12, cudaMemcpyHostToDevice, st);
			if (e == cudaSuccess) e = s->Eval(dp.As<float>(), n, 3, dout.As<float>(), st);
			if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout.Ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
			if (e == cudaSuccess) e = cudaStreamSynchronize(st);
			dp.Release();
			dout.Release();
		}
		if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the surrogate kernels"); return TG_ERR_CUDA; }
		return e == cudaSuccess ? TG_OK : CudaFail(e, "evaluating the surrogate");
	}

	TANGERINE_API tg_status tg_surrogate_gradients(tg_surrogate* s, const float* samples, int64_t n, float* table_grad, float* mlp_grad,
		float* loss)
	{
		if (!s || !samples || n <= 0) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = eng.DefaultStream();
		DeviceBuffer d;
		cudaError_t e = d.Reserve((size_t)n * 16);
		if (e == cudaSuccess) e = cudaMemcpyAsync(d.Ptr, samples, (size_t)n * 16, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = s->Gradients(d.As<float4>(), n, table_grad, mlp_grad, loss, st);
		d.Release();
		if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the surrogate kernels"); return TG_ERR_CUDA; }
		return e == cudaSuccess ? TG_OK : CudaFail(e, "surrogate gradients");
	}

	TANGERINE_API tg_status tg_surrogate_train(tg_surrogate* s, const float* samples, int64_t n, int steps, void* stream)
	{
		if (!s || !samples || n <= 0 || steps < 0) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = StreamOf(stream);
		DeviceBuffer d;
		cudaError_t e = d.Reserve((size_t)n * 16);
		if (e == cudaSuccess) e = cudaMemcpyAsync(d.Ptr, samples, (size_t)n * 16, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = s->Train(d.As<float4>(), n, steps, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		d.Release();
		if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the surrogate kernels"); return TG_ERR_CUDA; }
		return e == cudaSuccess ? TG_OK : CudaFail(e, "training the surrogate");
	}

	TANGERINE_API tg_status tg_surrogate_margin(const tg_surrogate* s, float radius, float* margin)
	{
		if (!s || !margin) { SetError("null argument"); return TG_ERR_INVALID; }
		*margin = s->MarginFor(radius);
		return TG_OK;
	}

	TANGERINE_API tg_status tg_surrogate_set_margin(tg_surrogate* s, float margin)
	{
		if (!s || margin != margin) { SetError("invalid argument"); return TG_ERR_INVALID; }
		s->Info.MarginOverride = margin >= 0.0f ? margin : -1.0f;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_export_mesh_surrogate_device(tg_program* p, tg_surrogate* sur, const tg_grid* g, uint32_t flags,
		tg_device_mesh* out, void* stream)
	{
		if (!p || !sur || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		if (flags & TG_MESH_DENSE) { SetError("the surrogate export culls bricks: TG_MESH_DENSE does not apply"); return TG_ERR_INVALID; }
		GridSpec gs;
		if (!ToGridSpec(g, gs)) return TG_ERR_INVALID;
		if (((flags >> 8) & 0xFFu) > 32) { SetError("brick size must be 1..32 cells"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		ExportOptions opt = OptionsOf(flags);
		opt.Field = sur;
		opt.Refine = (flags & TG_MESH_SURROGATE_ONLY) == 0;
		DeviceMesh dm;
		cudaError_t e = eng.Export(*p, gs, opt, dm, StreamOf(stream));
		if (e == cudaErrorLaunchTimeout) { SetError("a tensor-core wait timed out in the surrogate kernels"); return TG_ERR_CUDA; }
		if (e != cudaSuccess) return CudaFail(e, "exporting the mesh");
		out->vertex_count = dm.VertexCount;
		out->face_count = dm.FaceCount;
		out->vertices = dm.Vertices;
		out->normals = dm.Normals;
		out->colors = dm.Colors;
		out->faces = dm.Faces;
		out->cubes = dm.Cubes;
		return TG_OK;
	}

	TANGERINE_API tg_status tg_export_mesh_surrogate(tg_program* p, tg_surrogate* sur, const tg_grid* g, uint32_t flags, tg_mesh* out,
		void* stream)
	{
		if (!p || !sur || !out) { SetError("null argument"); return TG_ERR_INVALID; }
		if (flags & TG_MESH_DENSE) { SetError("the surrogate export culls bricks: TG_MESH_DENSE does not apply"); return TG_ERR_INVALID; }
		GridSpec gs;
		if (!ToGridSpec(g, gs)) return TG_ERR_INVALID;
		if (((flags >> 8) & 0xFFu) > 32) { SetError("brick size must be 1..32 cells"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t s = StreamOf(stream);
		ExportOptions opt = OptionsOf(flags);
		opt.Field = sur;
		opt.Refine = (flags & TG_MESH_SURROGATE_ONLY) == 0;
		DeviceMesh dm;
		HostMeshOut host;
		opt.Host = &host;
		cudaError_t e = eng.Export(*p, gs, opt, dm, s);
		if (e == cudaErrorLaunchTimeout)
		{
			FreeHostMesh(host);
			std::memset(out, 0, sizeof *out);
			SetError("a tensor-core wait timed out in the surrogate kernels");
			return TG_ERR_CUDA;
		}
		return TakeHostMesh(e, host, out, "exporting the mesh");
	}

	TANGERINE_API tg_status tg_debug_mma(int mode, const float* a, const float* b, float* d)
	{
		if (!a || !b || !d || mode < 0 || mode > 2) { SetError("invalid argument"); return TG_ERR_INVALID; }
		const size_t na = mode == 1 ? 128 * 128 : 128 * 64;
		const size_t nb = mode == 1 ? 128 * 144 : 64 * 64;
		const size_t nd = mode == 1 ? 128 * 144 : 128 * 64;
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = eng.DefaultStream();
		DeviceBuffer da, db, dd, ds;
		cudaError_t e = da.Reserve(na * 4);
		if (e == cudaSuccess) e = db.Reserve(nb * 4);
		if (e == cudaSuccess) e = dd.Reserve(nd * 4);
		if (e == cudaSuccess) e = ds.Reserve(4);
		if (e == cudaSuccess) e = cudaMemsetAsync(ds.Ptr, 0, 4, st);
		if (e == cudaSuccess) e = cudaMemsetAsync(dd.Ptr, 0, nd * 4, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(da.Ptr, a, na * 4, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(db.Ptr, b, nb * 4, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess) e = LaunchDebugMma(mode, da.As<float>(), db.As<float>(), dd.As<float>(), ds.As<int>(), st);
		int status = 0;
		if (e == cudaSuccess) e = cudaMemcpyAsync(d, dd.Ptr, nd * 4, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(&status, ds.Ptr, 4, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		da.Release(); db.Release(); dd.Release(); ds.Release();
		if (e != cudaSuccess) return CudaFail(e, "tensor-core layout check");
		if (status) { SetError("a tensor-core wait timed out"); return TG_ERR_CUDA; }
		return TG_OK;
	}

	TANGERINE_API int64_t tg_last_export_bricks(uint32_t* out, int64_t capacity, int* brick_size)
	{
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		std::vector<uint32_t> list;
		int b = 0;
		if (eng.LastBrickList(list, b) != cudaSuccess) { SetError("reading the brick list"); return -1; }
		if (brick_size) *brick_size = b;
		if (out)
			for (int64_t i = 0; i < capacity && i < (int64_t)list.size(); ++i) out[i] = list[(size_t)i];
		return (int64_t)list.size();
	}

	TANGERINE_API tg_status tg_debug_blend_check(uint64_t n, uint64_t seed, uint64_t* counts)
	{
		if (!counts) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = eng.DefaultStream();
		DeviceBuffer d;
		unsigned long long host[3] = { 0, 0, 0 };
		cudaError_t e = d.Reserve(3 * sizeof(unsigned long long));
		if (e == cudaSuccess) e = LaunchBlendCheck(n, seed, d.As<unsigned long long>(), st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(host, d.Ptr, sizeof host, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		d.Release();
		if (e != cudaSuccess) return CudaFail(e, "blend check");
		for (int i = 0; i < 3; ++i) counts[i] = host[i];
		return TG_OK;
	}

	TANGERINE_API tg_status tg_debug_pair_check(uint64_t n, uint64_t seed, uint64_t* counts)
	{
		if (!counts) { SetError("null argument"); return TG_ERR_INVALID; }
		Engine& eng = Engine::Get();
		std::lock_guard<std::mutex> lock(eng.Mutex);
		const cudaStream_t st = eng.DefaultStream();
		DeviceBuffer d;
		unsigned long long host[10] = {};
		cudaError_t e = d.Reserve(sizeof host);
		if (e == cudaSuccess) e = LaunchPairCheck(n, seed, d.As<unsigned long long>(), st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(host, d.Ptr, sizeof host, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		d.Release();
		if (e != cudaSuccess) return CudaFail(e, "paired arithmetic check");
		for (int i = 0; i < 10; ++i) counts[i] = host[i];
		return TG_OK;
	}

	TANGERINE_API const char* tg_last_error(void) { return LastError().c_str(); }
	TANGERINE_API const char* tg_version(void) { return "tangerine_gb300 0.1 (sm_103a)"; }
}
