// Test infrastructure only: a thin extern "C" harness over Tangerine's own CPU code,
// compiled together with the reference sources (tangerine/sdf_evaluator.cpp, export.cpp,
// third_party/naive-surface-nets, ...) by oracle/Makefile into oracle/_ref/.
// It is used to pin the C restatement in oracle/port and to write the golden fixtures
// under tests/golden.  Nothing in the product links or loads it.
//
// Trees are built from a "tree spec": a postfix word stream (float32 words, opcodes are
// small integers stored as floats) that is executed on a stack of SDFNodeShared using the
// reference's SDF:: constructors and SDFNode mutators (tangerine/sdf_evaluator.h:223-264).

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <chrono>
#include <fstream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sdf_evaluator.h"
#include "material.h"
#include "export.h"
#include "transform.h"
#include "magica.h"
#include <VoxWriter.h>
#include "painting_set.h"
#include "threadpool.h"
#include <surface_nets.h>
#include <set>

using namespace glm;

// painting_set.h declares this; the export path we call never uses it (MeshExport with
// an explicit evaluator does not read the painting set).
void PaintingSet::GlobalApply(std::function<void(SDFModelShared)>& Thunk) {}

// Globals owned by tangerine/export.cpp (export.cpp:48-57).
extern std::atomic_bool ExportActive;
extern std::atomic_int ExportState;
extern std::atomic_int VoxelCount;
extern std::atomic_int GenerationProgress;
extern std::atomic_int RefinementProgress;
extern std::atomic_int WriteProgress;
void MeshExportThread(SDFNodeShared Evaluator, vec3 ModelMin, vec3 ModelMax, vec3 Step, int RefineIterations, std::string Path, ExportFormat Format, float Scale);
void WritePLY(std::string Path, std::vector<vec3>& Vertices, std::vector<uint8_t>& Colors, std::vector<glm::vec3>& Normals, std::vector<ivec3>& Triangles);
void WriteSTL(std::string Path, std::vector<vec3>& Vertices, std::vector<glm::vec3>& Normals, std::vector<ivec3>& Triangles);
void PointCloudExportThread(SDFNodeShared Evaluator, vec3 ModelMin, vec3 ModelMax, vec3 Step, int RefineIterations, std::string Path, ExportFormat Format, float Scale);

namespace
{
	enum SpecOp
	{
		S_SPHERE = 1, S_ELLIPSOID, S_BOX, S_TORUS, S_CYLINDER, S_PLANE, S_CONE, S_CONINDER,
		S_UNION, S_DIFF, S_INTER, S_BUNION, S_BDIFF, S_BINTER, S_FLATE,
		S_MOVE, S_ROTATE, S_SCALE, S_PAINT, S_ALIGN, S_STENCIL,
	};

	struct RefTree
	{
		SDFNodeShared Root;
	};

	struct RefOctree
	{
		SDFOctreeShared Octree;
	};

	int Arity(int Op)
	{
		switch (Op)
		{
		case S_SPHERE: return 1;
		case S_ELLIPSOID: case S_BOX: case S_PLANE: return 3;
		case S_TORUS: case S_CYLINDER: case S_CONE: return 2;
		case S_CONINDER: return 3;
		case S_UNION: case S_DIFF: case S_INTER: return 0;
		case S_BUNION: case S_BDIFF: case S_BINTER: case S_FLATE: return 1;
		case S_MOVE: return 3;
		case S_ROTATE: return 4;
		case S_SCALE: return 1;
		case S_PAINT: return 3;
		case S_ALIGN: return 3;
		case S_STENCIL: return 4;
		default: return -1;
		}
	}

	SDFNodeShared BuildSpec(const float* Spec, int Count)
	{
		std::vector<SDFNodeShared> Stack;
		int i = 0;
		while (i < Count)
		{
			const int Op = (int)Spec[i++];
			const int N = Arity(Op);
			if (N < 0 || i + N > Count)
			{
				return nullptr;
			}
			const float* P = Spec + i;
			i += N;
			auto Pop = [&]() -> SDFNodeShared
			{
				SDFNodeShared Top = Stack.back();
				Stack.pop_back();
				return Top;
			};
			switch (Op)
			{
			case S_SPHERE: Stack.push_back(SDF::Sphere(P[0])); break;
			case S_ELLIPSOID: Stack.push_back(SDF::Ellipsoid(P[0], P[1], P[2])); break;
			case S_BOX: Stack.push_back(SDF::Box(P[0], P[1], P[2])); break;
			case S_TORUS: Stack.push_back(SDF::Torus(P[0], P[1])); break;
			case S_CYLINDER: Stack.push_back(SDF::Cylinder(P[0], P[1])); break;
			case S_PLANE: Stack.push_back(SDF::Plane(P[0], P[1], P[2])); break;
			case S_CONE: Stack.push_back(SDF::Cone(P[0], P[1])); break;
			case S_CONINDER: Stack.push_back(SDF::Coninder(P[0], P[1], P[2])); break;
			case S_UNION: case S_DIFF: case S_INTER:
			case S_BUNION: case S_BDIFF: case S_BINTER:
			{
				if (Stack.size() < 2) return nullptr;
				SDFNodeShared RHS = Pop();
				SDFNodeShared LHS = Pop();
				SDFNodeShared Out;
				if (Op == S_UNION) Out = SDF::Union(LHS, RHS);
				else if (Op == S_DIFF) Out = SDF::Diff(LHS, RHS);
				else if (Op == S_INTER) Out = SDF::Inter(LHS, RHS);
				else if (Op == S_BUNION) Out = SDF::BlendUnion(P[0], LHS, RHS);
				else if (Op == S_BDIFF) Out = SDF::BlendDiff(P[0], LHS, RHS);
				else Out = SDF::BlendInter(P[0], LHS, RHS);
				Stack.push_back(Out);
				break;
			}
			case S_FLATE:
			{
				if (Stack.empty()) return nullptr;
				SDFNodeShared Child = Pop();
				Stack.push_back(SDF::Flate(Child, P[0]));
				break;
			}
			case S_MOVE:
				if (Stack.empty()) return nullptr;
				Stack.back()->Move(vec3(P[0], P[1], P[2]));
				break;
			case S_ROTATE:
				// Same argument order as RotateTree (c_sdf.cpp:93-98): quat(W, X, Y, Z).
				if (Stack.empty()) return nullptr;
				Stack.back()->Rotate(quat(P[3], P[0], P[1], P[2]));
				break;
			case S_SCALE:
				if (Stack.empty()) return nullptr;
				Stack.back()->Scale(P[0]);
				break;
			case S_PAINT:
			{
				if (Stack.empty()) return nullptr;
				MaterialShared Material = MaterialShared(new MaterialPBRBR(ColorPoint(vec3(P[0], P[1], P[2]))));
				Stack.back()->ApplyMaterial(Material, false);
				break;
			}
			case S_ALIGN:
				if (Stack.empty()) return nullptr;
				SDF::Align(Stack.back(), vec3(P[0], P[1], P[2]));
				break;
			case S_STENCIL:
			{
				if (Stack.size() < 2) return nullptr;
				SDFNodeShared Mask = Pop();
				SDFNodeShared Node = Pop();
				MaterialShared Material = MaterialShared(new MaterialPBRBR(ColorPoint(vec3(P[1], P[2], P[3]))));
				Stack.push_back(SDF::Stencil(Node, Mask, Material, P[0] != 0.0f));
				break;
			}
			default:
				return nullptr;
			}
		}
		if (Stack.size() != 1)
		{
			return nullptr;
		}
		return Stack.back();
	}

	void ColorBytes(MaterialShared Material, uint8_t* Out)
	{
		// Same arithmetic as WritePLY(Octree, ...) (export.cpp:303-311).
		vec3 Color = vec3(1.0f);
		if (Material)
		{
			Color = SampleColor(Material->GuessColor());
		}
		Out[0] = 0xFF * Color.r;
		Out[1] = 0xFF * Color.g;
		Out[2] = 0xFF * Color.b;
	}

	struct OctreeDump
	{
		std::vector<float> Nodes;        // per node: pivot xyz, bounds min xyz, max xyz, terminus, has_eval, program offset, program length, stack size
		std::vector<int32_t> Children;   // per node: 8 child indices (-1 = none)
		std::vector<uint32_t> Words;     // concatenated programs
	};

	int DumpNode(SDFOctree* Node, OctreeDump& Out)
	{
		const int Index = (int)(Out.Children.size() / 8);
		for (int c = 0; c < 8; ++c) Out.Children.push_back(-1);
		const size_t Base = Out.Nodes.size();
		Out.Nodes.resize(Base + 14);
		float* N = &Out.Nodes[Base];
		N[0] = Node->Pivot.x; N[1] = Node->Pivot.y; N[2] = Node->Pivot.z;
		N[3] = Node->Bounds.Min.x; N[4] = Node->Bounds.Min.y; N[5] = Node->Bounds.Min.z;
		N[6] = Node->Bounds.Max.x; N[7] = Node->Bounds.Max.y; N[8] = Node->Bounds.Max.z;
		N[9] = Node->Terminus ? 1.0f : 0.0f;
		N[10] = Node->Evaluator ? 1.0f : 0.0f;
		N[11] = (float)Out.Words.size();
		N[12] = 0.0f;
		N[13] = 0.0f;
		if (Node->Interpreter)
		{
			const ProgramBuffer& Program = Node->Interpreter->Program;
			for (size_t w = 0; w < Program.Size(); ++w)
			{
				uint32_t Bits;
				std::memcpy(&Bits, &Program.Words[w], 4);
				Out.Words.push_back(Bits);
			}
			Out.Nodes[Base + 12] = (float)Program.Size();
			Out.Nodes[Base + 13] = (float)Node->Interpreter->StackSize;
		}
		if (!Node->Terminus)
		{
			for (int c = 0; c < 8; ++c)
			{
				if (Node->Children[c])
				{
					const int ChildIndex = DumpNode(Node->Children[c], Out);
					Out.Children[Index * 8 + c] = ChildIndex;
				}
			}
		}
		return Index;
	}

	template<typename T>
	T* CopyOut(const std::vector<T>& In)
	{
		T* Out = (T*)std::malloc(std::max<size_t>(1, In.size()) * sizeof(T));
		if (!In.empty()) std::memcpy(Out, In.data(), In.size() * sizeof(T));
		return Out;
	}

	struct MeshOut
	{
		std::vector<float> Vertices;
		std::vector<uint64_t> CubeOfVertex;
		std::vector<uint64_t> Faces;
	};
}

extern "C"
{
	void* ref_build(const float* Spec, int Count)
	{
		SDFNodeShared Root = BuildSpec(Spec, Count);
		if (!Root) return nullptr;
		return new RefTree{ Root };
	}

	void ref_free(void* Handle)
	{
		delete (RefTree*)Handle;
	}

	void ref_free_buffer(void* Buffer)
	{
		std::free(Buffer);
	}

	int ref_stack_size(void* Handle)
	{
		return (int)((RefTree*)Handle)->Root->StackSize;
	}

	int ref_has_paint(void* Handle)
	{
		return ((RefTree*)Handle)->Root->HasPaint() ? 1 : 0;
	}

	int ref_has_finite_bounds(void* Handle)
	{
		return ((RefTree*)Handle)->Root->HasFiniteBounds() ? 1 : 0;
	}

	int ref_leaf_count(void* Handle)
	{
		return ((RefTree*)Handle)->Root->LeafCount();
	}

	void ref_bounds(void* Handle, float* Out, int Inner)
	{
		SDFNodeShared& Root = ((RefTree*)Handle)->Root;
		AABB B = Inner ? Root->InnerBounds() : Root->Bounds();
		Out[0] = B.Min.x; Out[1] = B.Min.y; Out[2] = B.Min.z;
		Out[3] = B.Max.x; Out[4] = B.Max.y; Out[5] = B.Max.z;
	}

	// Virtual SDFNode::Eval over n points.
	void ref_eval(void* Handle, int64_t Count, const float* Points, float* Out)
	{
		SDFNodeShared& Root = ((RefTree*)Handle)->Root;
		for (int64_t i = 0; i < Count; ++i)
		{
			Out[i] = Root->Eval(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2]));
		}
	}

	void ref_gradient(void* Handle, int64_t Count, const float* Points, float* Out)
	{
		SDFNodeShared& Root = ((RefTree*)Handle)->Root;
		for (int64_t i = 0; i < Count; ++i)
		{
			vec3 G = Root->Gradient(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2]));
			Out[i * 3 + 0] = G.x; Out[i * 3 + 1] = G.y; Out[i * 3 + 2] = G.z;
		}
	}

	void ref_color(void* Handle, int64_t Count, const float* Points, uint8_t* Out)
	{
		SDFNodeShared& Root = ((RefTree*)Handle)->Root;
		for (int64_t i = 0; i < Count; ++i)
		{
			ColorBytes(Root->GetMaterial(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2])), Out + i * 3);
		}
	}

	// Full-tree program words (SDFInterpreter ctor, sdf_evaluator.cpp:1376-1383).
	int ref_compile(void* Handle, uint32_t* Out, int Capacity)
	{
		SDFInterpreter Interpreter(((RefTree*)Handle)->Root);
		const int Size = (int)Interpreter.Program.Size();
		for (int i = 0; i < Size && i < Capacity; ++i)
		{
			std::memcpy(&Out[i], &Interpreter.Program.Words[i], 4);
		}
		return Size;
	}

	void ref_interp_eval(void* Handle, int64_t Count, const float* Points, float* Out)
	{
		SDFInterpreter Interpreter(((RefTree*)Handle)->Root);
		for (int64_t i = 0; i < Count; ++i)
		{
			Out[i] = Interpreter.Eval(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2]));
		}
	}

	void* ref_clip(void* Handle, float X, float Y, float Z, float Radius)
	{
		SDFNodeShared Clipped = ((RefTree*)Handle)->Root->Clip(vec3(X, Y, Z), Radius);
		if (!Clipped) return nullptr;
		return new RefTree{ Clipped };
	}

	int ref_equal(void* A, void* B)
	{
		return (*((RefTree*)A)->Root == *((RefTree*)B)->Root) ? 1 : 0;
	}

	void* ref_octree_create(void* Handle, float TargetSize, int Coalesce, int MaxDepth)
	{
		SDFOctreeShared Octree = SDFOctree::Create(((RefTree*)Handle)->Root, TargetSize, Coalesce != 0, MaxDepth);
		if (!Octree) return nullptr;
		return new RefOctree{ Octree };
	}

	// Sodapop's meshing octree (sodapop.cpp:565-569): Create(.25, false, 3), then every
	// incomplete cell populated with Populate(false, 3, -1).
	void* ref_meshing_octree_create(void* Handle)
	{
		SDFOctreeShared Octree = SDFOctree::Create(((RefTree*)Handle)->Root, .25, false, 3, 0.0f);
		if (!Octree) return nullptr;
		std::vector<SDFOctree*> Incompletes;
		SDFOctree::CallbackType Search = [&](SDFOctree& Leaf)
		{
			if (Leaf.Incomplete) Incompletes.push_back(&Leaf);
		};
		Octree->Walk(Search);
		for (SDFOctree* Cell : Incompletes) Cell->Populate(false, 3, -1);
		return new RefOctree{ Octree };
	}

	void ref_octree_free(void* Handle)
	{
		delete (RefOctree*)Handle;
	}

	// Dumps the octree in depth-first order.  Returns the node count; the three buffers
	// are malloc'd and must be released with ref_free_buffer.
	int ref_octree_dump(void* Handle, float** Nodes, int32_t** Children, uint32_t** Words, int* WordCount)
	{
		OctreeDump Dump;
		DumpNode(((RefOctree*)Handle)->Octree.get(), Dump);
		*Nodes = CopyOut(Dump.Nodes);
		*Children = CopyOut(Dump.Children);
		*Words = CopyOut(Dump.Words);
		*WordCount = (int)Dump.Words.size();
		return (int)(Dump.Children.size() / 8);
	}

	void ref_octree_eval(void* Handle, int64_t Count, const float* Points, int Exact, float* Out)
	{
		SDFOctreeShared& Octree = ((RefOctree*)Handle)->Octree;
		for (int64_t i = 0; i < Count; ++i)
		{
			Out[i] = Octree->Eval(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2]), Exact != 0);
		}
	}

	// Evaluates SDFOctree::Eval(p, Exact=true) on the export lattice
	// p = (x0 + i*dx, y0 + j*dy, z0 + k*dz), i fastest, using all host threads.
	void ref_octree_grid(void* Handle, float X0, float Y0, float Z0, float DX, float DY, float DZ,
		int64_t NX, int64_t NY, int64_t NZ, float* Out)
	{
		SDFOctreeShared& Octree = ((RefOctree*)Handle)->Octree;
		std::atomic<int64_t> NextSlice(0);
		Pool([&]()
		{
			for (int64_t k = NextSlice.fetch_add(1); k < NZ; k = NextSlice.fetch_add(1))
			{
				const float Z = Z0 + static_cast<float>(k) * DZ;
				for (int64_t j = 0; j < NY; ++j)
				{
					const float Y = Y0 + static_cast<float>(j) * DY;
					for (int64_t i = 0; i < NX; ++i)
					{
						const float X = X0 + static_cast<float>(i) * DX;
						Out[(k * NY + j) * NX + i] = Octree->Eval(vec3(X, Y, Z));
					}
				}
			}
		});
	}

	void ref_octree_gradient(void* Handle, int64_t Count, const float* Points, float* Out)
	{
		SDFOctreeShared& Octree = ((RefOctree*)Handle)->Octree;
		for (int64_t i = 0; i < Count; ++i)
		{
			vec3 G = Octree->Gradient(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2]));
			Out[i * 3 + 0] = G.x; Out[i * 3 + 1] = G.y; Out[i * 3 + 2] = G.z;
		}
	}

	void ref_octree_color(void* Handle, int64_t Count, const float* Points, uint8_t* Out)
	{
		SDFOctreeShared& Octree = ((RefOctree*)Handle)->Octree;
		for (int64_t i = 0; i < Count; ++i)
		{
			ColorBytes(Octree->GetMaterial(vec3(Points[i * 3 + 0], Points[i * 3 + 1], Points[i * 3 + 2])), Out + i * 3);
		}
	}

	// Octree->Evaluator->HasPaint(): WritePLY(Octree, ...) writes colours (export.cpp:285).
	int ref_octree_has_paint(void* Handle)
	{
		return ((RefOctree*)Handle)->Octree->Evaluator->HasPaint() ? 1 : 0;
	}

	// WritePLY(Octree, ...)'s per-vertex attribute loop (export.cpp:283-317: Gradient, then
	// GetMaterial -> SampleColor -> 0xFF * c when the tree has paint) over Pool() threads
	// (Threads <= 0) or `Threads` threads, vertices handed out in order.  Colors may be null.
	void ref_vertex_attributes(void* Handle, int64_t Count, const float* Points, int Threads, float* Normals, uint8_t* Colors)
	{
		SDFOctreeShared Octree = ((RefOctree*)Handle)->Octree;
		std::atomic<int64_t> Next(0);
		auto Thunk = [&]()
		{
			for (int64_t i = Next.fetch_add(256); i < Count; i = Next.fetch_add(256))
			{
				const int64_t End = std::min<int64_t>(Count, i + 256);
				for (int64_t v = i; v < End; ++v)
				{
					const vec3 P(Points[v * 3 + 0], Points[v * 3 + 1], Points[v * 3 + 2]);
					const vec3 G = Octree->Gradient(P);
					Normals[v * 3 + 0] = G.x; Normals[v * 3 + 1] = G.y; Normals[v * 3 + 2] = G.z;
					if (Colors) ColorBytes(Octree->GetMaterial(P), Colors + v * 3);
				}
			}
		};
		if (Threads <= 0)
		{
			Pool(Thunk);
		}
		else
		{
			std::vector<std::thread> Workers;
			for (int t = 0; t < Threads; ++t) Workers.emplace_back(Thunk);
			for (auto& W : Workers) W.join();
		}
	}

	// Runs Tangerine's naive surface nets (the AsyncParallelSurfaceNets thunks that
	// par_surface_nets drives, surface_nets.cpp:1148-1205) over the export octree, with
	// the z-slices and then the active-cell map entries spread over Pool() threads.
	// Returns the vertex count; vertex positions (3 floats each), the active cube index of
	// each vertex and the faces (3 vertex indices each) are malloc'd.
	int64_t ref_surface_nets(void* Handle, float X0, float Y0, float Z0, float DX, float DY, float DZ,
		int64_t SX, int64_t SY, int64_t SZ, int Threads,
		float** Vertices, uint64_t** Cubes, uint64_t** Faces, int64_t* FaceCount, double* Seconds)
	{
		SDFOctreeShared Octree = ((RefOctree*)Handle)->Octree;
		auto Start = std::chrono::steady_clock::now();

		isosurface::AsyncParallelSurfaceNets Task;
		Task.ImplicitFunction = [Octree](float X, float Y, float Z) -> float
		{
			return Octree->Eval(vec3(X, Y, Z));
		};
		Task.Grid.x = X0; Task.Grid.y = Y0; Task.Grid.z = Z0;
		Task.Grid.dx = DX; Task.Grid.dy = DY; Task.Grid.dz = DZ;
		Task.Grid.sx = SX; Task.Grid.sy = SY; Task.Grid.sz = SZ;
		Task.Setup();

		auto RunThreads = [&](const std::function<void()>& Thunk)
		{
			if (Threads <= 0)
			{
				Pool(Thunk);
			}
			else
			{
				std::vector<std::thread> Workers;
				for (int t = 0; t < Threads; ++t) Workers.emplace_back(Thunk);
				for (auto& W : Workers) W.join();
			}
		};

		std::atomic<size_t> Next(0);
		RunThreads([&]()
		{
			for (size_t n = Next.fetch_add(1); n < Task.FirstLoopDomain.size(); n = Next.fetch_add(1))
			{
				Task.FirstLoopThunk(Task, Task.FirstLoopDomain[n]);
			}
		});

		std::vector<std::pair<const size_t, uint64_t>*> Entries;
		Entries.reserve(Task.SecondLoopDomain.size());
		for (auto& Entry : Task.SecondLoopDomain) Entries.push_back(&Entry);
		Next.store(0);
		RunThreads([&]()
		{
			for (size_t n = Next.fetch_add(1); n < Entries.size(); n = Next.fetch_add(1))
			{
				Task.SecondLoopThunk(Task, *Entries[n]);
			}
		});

		*Seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - Start).count();

		const size_t VertexCount = Task.OutputMesh.vertices_.size();
		std::vector<float> V(VertexCount * 3);
		std::vector<uint64_t> C(VertexCount, ~uint64_t(0));
		for (size_t v = 0; v < VertexCount; ++v)
		{
			V[v * 3 + 0] = Task.OutputMesh.vertices_[v].x;
			V[v * 3 + 1] = Task.OutputMesh.vertices_[v].y;
			V[v * 3 + 2] = Task.OutputMesh.vertices_[v].z;
		}
		for (auto& Entry : Task.SecondLoopDomain)
		{
			C[Entry.second] = Entry.first;
		}
		std::vector<uint64_t> F;
		F.reserve(Task.OutputMesh.faces_.size() * 3);
		for (auto& Face : Task.OutputMesh.faces_)
		{
			F.push_back(Face.v0); F.push_back(Face.v1); F.push_back(Face.v2);
		}
		*Vertices = CopyOut(V);
		*Cubes = CopyOut(C);
		*Faces = CopyOut(F);
		*FaceCount = (int64_t)Task.OutputMesh.faces_.size();
		return (int64_t)VertexCount;
	}

	// MeshingJob::NaiveSurfaceNets (sodapop.cpp:562-897) replayed serially with the
	// reference's own classes: the meshing octree (SDFOctree::Create(.25, no coalescing,
	// depth 3), then every incomplete cell populated without limit, LinkLeaves), the grid of
	// NaiveSurfaceNetsScratch (sodapop.cpp:150-177), the point cache over the leaves' aligned
	// boxes, FirstLoopInnerThunk for each cached point in index order (the std::set order of
	// each bucket, buckets in order), SecondLoopThunk for each map entry, then per vertex
	// SDFOctree::Gradient and the material's Eval with the normal as the view direction
	// (sodapop.cpp:815-872).  Left out: ApplyVertexSequence's shuffle, whose input order is
	// already run-dependent in the app (parallel vertex loop).  Returns the vertex count
	// (-1 without an octree); grid_out receives x, y, z, dx, dy, dz, sx, sy, sz.
	int64_t ref_sodapop(void* Handle, float Density, float** Positions, float** Normals, float** Colors, uint64_t** Faces,
		int64_t* FaceCount, float* GridOut)
	{
		SDFNodeShared Root = ((RefTree*)Handle)->Root;
		SDFOctreeShared Evaluator = SDFOctree::Create(Root, .25, false, 3, 0.0f);
		if (!Evaluator) return -1;
		std::vector<SDFOctree*> Incompletes;
		SDFOctree::CallbackType Search = [&](SDFOctree& Leaf)
		{
			if (Leaf.Incomplete) Incompletes.push_back(&Leaf);
		};
		Evaluator->Walk(Search);
		for (SDFOctree* Cell : Incompletes) Cell->Populate(false, 3, -1);
		Evaluator->LinkLeaves();

		isosurface::AsyncParallelSurfaceNets Ext;
		isosurface::regular_grid_t& Grid = Ext.Grid;
		{
			const float Floored = glm::floor(Density);
			const glm::vec3 SamplesPerUnit = glm::max(Evaluator->Bounds.Extent() * glm::vec3(Floored), glm::vec3(8.0));
			Grid.x = Evaluator->Bounds.Min.x;
			Grid.y = Evaluator->Bounds.Min.y;
			Grid.z = Evaluator->Bounds.Min.z;
			Grid.sx = size_t(glm::ceil(SamplesPerUnit.x));
			Grid.sy = size_t(glm::ceil(SamplesPerUnit.y));
			Grid.sz = size_t(glm::ceil(SamplesPerUnit.z));
			Grid.dx = Evaluator->Bounds.Extent().x / static_cast<float>(Grid.sx);
			Grid.dy = Evaluator->Bounds.Extent().y / static_cast<float>(Grid.sy);
			Grid.dz = Evaluator->Bounds.Extent().z / static_cast<float>(Grid.sz);
			Grid.x -= Grid.dx * 2;
			Grid.y -= Grid.dy * 2;
			Grid.z -= Grid.dz * 2;
			Grid.sx += 3;
			Grid.sy += 3;
			Grid.sz += 3;
		}
		GridOut[0] = Grid.x; GridOut[1] = Grid.y; GridOut[2] = Grid.z;
		GridOut[3] = Grid.dx; GridOut[4] = Grid.dy; GridOut[5] = Grid.dz;
		GridOut[6] = (float)Grid.sx; GridOut[7] = (float)Grid.sy; GridOut[8] = (float)Grid.sz;
		SDFOctree* Raw = Evaluator.get();
		Ext.ImplicitFunction = [Raw](float X, float Y, float Z) -> float
		{
			return glm::clamp(Raw->Eval(glm::vec3(X, Y, Z), false), -100.0f, 100.0f);
		};
		Ext.Setup();

		const size_t IndexRange = Grid.sx * Grid.sy * Grid.sz;
		const size_t BucketSize = std::min(size_t(64), IndexRange);
		const size_t BucketCount = (IndexRange + BucketSize - 1) / BucketSize;
		std::set<size_t> Points;
		{
			const glm::vec3 Origin(Grid.x, Grid.y, Grid.z);
			const glm::vec3 Step(Grid.dx, Grid.dy, Grid.dz);
			for (SDFOctree* Leaf = Evaluator->Next; Leaf; Leaf = (Leaf->Next == Leaf ? nullptr : Leaf->Next))
			{
				const glm::vec3 AlignedMin = glm::floor(glm::max(glm::vec3(0.0), Leaf->Bounds.Min - Origin) / Step);
				const glm::vec3 AlignedMax = glm::ceil((Leaf->Bounds.Max - Origin) / Step);
				for (float z = AlignedMin.z; z <= AlignedMax.z; ++z)
					for (float y = AlignedMin.y; y <= AlignedMax.y; ++y)
						for (float x = AlignedMin.x; x <= AlignedMax.x; ++x)
						{
							const size_t Index = size_t(x) + (size_t(y) * Grid.sx) + (size_t(z) * Grid.sx * Grid.sy);
							if (Index / BucketSize < BucketCount) Points.insert(Index);
						}
			}
		}
		for (size_t Index : Points)
		{
			isosurface::AsyncParallelSurfaceNets::GridPoint P;
			P.i = Index % Grid.sx;
			P.j = (Index / Grid.sx) % Grid.sy;
			P.k = Index / (Grid.sx * Grid.sy);
			Ext.FirstLoopInnerThunk(Ext, P);
		}
		for (auto& Element : Ext.SecondLoopDomain) Ext.SecondLoopThunk(Ext, Element);

		const size_t VertexCount = Ext.OutputMesh.vertices_.size();
		std::vector<float> P3(VertexCount * 3), N3(VertexCount * 3), C4(VertexCount * 4);
		for (size_t v = 0; v < VertexCount; ++v)
		{
			const glm::vec3 Position(Ext.OutputMesh.vertices_[v].x, Ext.OutputMesh.vertices_[v].y, Ext.OutputMesh.vertices_[v].z);
			P3[v * 3] = Position.x; P3[v * 3 + 1] = Position.y; P3[v * 3 + 2] = Position.z;
			const glm::vec3 Normal = Evaluator->Gradient(Position);
			N3[v * 3] = Normal.x; N3[v * 3 + 1] = Normal.y; N3[v * 3 + 2] = Normal.z;
			glm::vec3 Sample(0.0f);
			MaterialShared Material = Evaluator->GetMaterial(Position);
			if (Material)
			{
				ChthonicMaterialInterface* Chthonic = dynamic_cast<ChthonicMaterialInterface*>(Material.get());
				if (Chthonic) Sample = glm::vec3(Chthonic->Eval(Position, Normal, Normal));
			}
			C4[v * 4] = Sample.x; C4[v * 4 + 1] = Sample.y; C4[v * 4 + 2] = Sample.z; C4[v * 4 + 3] = 1.0f;
		}
		std::vector<uint64_t> F;
		F.reserve(Ext.OutputMesh.faces_.size() * 3);
		for (auto& Face : Ext.OutputMesh.faces_)
		{
			F.push_back(Face.v0); F.push_back(Face.v1); F.push_back(Face.v2);
		}
		*Positions = CopyOut(P3);
		*Normals = CopyOut(N3);
		*Colors = CopyOut(C4);
		*Faces = CopyOut(F);
		*FaceCount = (int64_t)Ext.OutputMesh.faces_.size();
		return (int64_t)VertexCount;
	}

	// The reference's own export entry (export.cpp:320-381) writing a PLY or STL file:
	// octree, surface nets, gradient normals, material colours, writer.
	void ref_mesh_export_file(void* Handle, float MinX, float MinY, float MinZ, float MaxX, float MaxY, float MaxZ,
		float Step, int Format, const char* Path)
	{
		ExportActive.store(true);
		ExportState.store(1);
		GenerationProgress.store(0);
		RefinementProgress.store(0);
		WriteProgress.store(0);
		MeshExportThread(((RefTree*)Handle)->Root, vec3(MinX, MinY, MinZ), vec3(MaxX, MaxY, MaxZ), vec3(Step), 0,
			std::string(Path), Format == 0 ? ExportFormat::STL : ExportFormat::PLY, 1.0f);
	}

	// The reference's point-cloud export (export.cpp:384-480) writing a PLY file.  Its
	// threads push points in a run-dependent order; every row is a function of its cell.
	void ref_point_cloud_file(void* Handle, const float* Min, const float* Max, const float* Step, int RefineIterations,
		float Scale, const char* Path)
	{
		ExportActive.store(true);
		ExportState.store(1);
		GenerationProgress.store(0);
		RefinementProgress.store(0);
		WriteProgress.store(0);
		PointCloudExportThread(((RefTree*)Handle)->Root, vec3(Min[0], Min[1], Min[2]), vec3(Max[0], Max[1], Max[2]),
			vec3(Step[0], Step[1], Step[2]), RefineIterations, std::string(Path), ExportFormat::PLY, Scale);
	}

	// The reference's MagicaVoxel export (magica.cpp:27-72) as shipped: threads add voxels in a
	// run-dependent order, which moves cubes and one translation in the file.
	void ref_vox_file(void* Handle, float GridSize, int ColorIndex, const char* Path)
	{
		std::string P(Path);
		VoxExport(((RefTree*)Handle)->Root, P, GridSize, ColorIndex);
	}

	// VoxExport's loop (magica.cpp:29-69) run serially in cell order, through the same
	// VoxWriter, so the file bytes are deterministic.  Returns the voxel count; Voxels gets
	// x, y, z, colour index per voxel (malloc'd) and Size the lattice.
	int64_t ref_vox_serial(void* Handle, float GridSize, int ColorIndex, const char* Path, int32_t** Voxels, int32_t* SizeOut,
		float* RadiusOut)
	{
		SDFNodeShared Evaluator = ((RefTree*)Handle)->Root;
		AABB Bounds = Evaluator->Bounds();
		glm::ivec3 Size = glm::ivec3(glm::ceil(Bounds.Max - Bounds.Min) * GridSize);
		float Radius;
		{
			glm::vec3 Alpha = glm::vec3(.5, .5, .5) / glm::vec3(Size);
			Radius = glm::distance(Bounds.Min, glm::mix(Bounds.Min, Bounds.Max, Alpha));
		}
		const int Slice = Size.x * Size.y;
		const int TotalCells = Size.x * Size.y * Size.z;
		vox::VoxWriter Writer(Size.x, Size.y, Size.z);
		std::vector<int32_t> Out;
		for (int i = 0; i < TotalCells; ++i)
		{
			int z = i / Slice;
			int y = (i % Slice) / Size.x;
			int x = i % Size.x;
			glm::vec3 Alpha = glm::vec3(x + .5, y + .5, z + .5) / glm::vec3(Size);
			glm::vec3 Point = glm::mix(Bounds.Min, Bounds.Max, Alpha);
			float Dist = Evaluator->Eval(Point);
			if (std::abs(Dist) <= Radius)
			{
				const int Color = abs(ColorIndex) % 255 + 1;
				Writer.AddVoxel(x, y, z, Color);
				Out.push_back(x); Out.push_back(y); Out.push_back(z); Out.push_back(Color);
			}
		}
		if (Path && Path[0]) Writer.SaveToFile(std::string(Path));
		*Voxels = CopyOut(Out);
		SizeOut[0] = Size.x; SizeOut[1] = Size.y; SizeOut[2] = Size.z;
		*RadiusOut = Radius;
		return (int64_t)(Out.size() / 4);
	}

	// VoxWriter given voxels (x, y, z, colour) in order, for checking a writer on volumes
	// larger than one 126-voxel cube.
	void ref_vox_write(const int32_t* Voxels, int64_t Count, const int32_t* Size, const char* Path)
	{
		vox::VoxWriter Writer(Size[0], Size[1], Size[2]);
		for (int64_t v = 0; v < Count; ++v)
		{
			Writer.AddVoxel(Voxels[v * 4], Voxels[v * 4 + 1], Voxels[v * 4 + 2], (uint8_t)Voxels[v * 4 + 3]);
		}
		Writer.SaveToFile(std::string(Path));
	}

	// The two framed ray casts of the app, serially: Mode 1 is Lua's magnet cast
	// (lua_sdf.cpp:410-417: Direction = normalize(Target - Origin), 100 iterations, 0.001 by
	// default); Mode 2 is SDFModel::RayMarch (sdf_model.cpp:261-266: the ray taken into the
	// model's frame, Transform{Rotation = quat(Q[0..3] as w x y z), Translation = T,
	// Scalation = S}, then 1000 iterations at the default epsilon).
	void ref_ray_query(void* Handle, int Mode, const float* Frame, int64_t Count, const float* Origins, const float* Dirs,
		int MaxIterations, float Epsilon, uint8_t* Hit, float* Travel, float* Position)
	{
		SDFNodeShared Root = ((RefTree*)Handle)->Root;
		Transform LocalToWorld;
		if (Mode == 2)
		{
			LocalToWorld.Rotation = glm::quat(Frame[0], Frame[1], Frame[2], Frame[3]);
			LocalToWorld.Translation = vec3(Frame[4], Frame[5], Frame[6]);
			LocalToWorld.Scalation = Frame[7];
		}
		for (int64_t r = 0; r < Count; ++r)
		{
			vec3 Origin(Origins[r * 3], Origins[r * 3 + 1], Origins[r * 3 + 2]);
			vec3 Direction(Dirs[r * 3], Dirs[r * 3 + 1], Dirs[r * 3 + 2]);
			RayHit H;
			if (Mode == 1)
			{
				Direction = glm::normalize(Direction - Origin);
				H = Root->RayMarch(Origin, Direction, MaxIterations, Epsilon);
			}
			else
			{
				vec3 RelativeOrigin = LocalToWorld.ApplyInv(Origin);
				vec3 RelativeRayDir = glm::rotate(glm::inverse(LocalToWorld.Rotation), Direction);
				H = Root->RayMarch(RelativeOrigin, RelativeRayDir, 1000);
			}
			Hit[r] = H.Hit ? 1 : 0;
			Travel[r] = H.Travel;
			Position[r * 3 + 0] = H.Position.x;
			Position[r * 3 + 1] = H.Position.y;
			Position[r * 3 + 2] = H.Position.z;
		}
	}

	// MeshExport(Path, UseBaseColor = true, ...)'s gather (export.cpp:495-548) over drawables
	// given as arrays (positions xyz, normals xyz, colours rgba, indices, per drawable), with
	// each model's LocalToWorld from a Transform {quat w x y z, translation, scale}, then the
	// reference's own writers.
	void ref_write_drawables(int Count, const int64_t* VertexCounts, const int64_t* IndexCounts, const float* Positions,
		const float* Normals, const float* Colors, const uint32_t* Indices, const float* Frames, int Format, float Scale,
		const char* Path)
	{
		std::vector<vec3> Vertices;
		std::vector<vec3> OutNormals;
		std::vector<uint8_t> OutColors;
		std::vector<ivec3> Triangles;
		size_t Offset = 0, IndexBase = 0;
		for (int d = 0; d < Count; ++d)
		{
			Transform LocalToWorldT;
			LocalToWorldT.Rotation = glm::quat(Frames[d * 8], Frames[d * 8 + 1], Frames[d * 8 + 2], Frames[d * 8 + 3]);
			LocalToWorldT.Translation = vec3(Frames[d * 8 + 4], Frames[d * 8 + 5], Frames[d * 8 + 6]);
			LocalToWorldT.Scalation = Frames[d * 8 + 7];
			glm::mat4 LocalToWorld = LocalToWorldT.ToMatrix();
			for (int64_t i = 0; i < VertexCounts[d]; ++i)
			{
				const size_t v = Offset + (size_t)i;
				const glm::vec4 Position(Positions[v * 3], Positions[v * 3 + 1], Positions[v * 3 + 2], 1.0);
				Vertices.push_back((LocalToWorld * Position).xyz() * glm::vec3(Scale));
				OutNormals.push_back(vec3(Normals[v * 3], Normals[v * 3 + 1], Normals[v * 3 + 2]));
				const glm::vec4 Color(Colors[v * 4], Colors[v * 4 + 1], Colors[v * 4 + 2], Colors[v * 4 + 3]);
				OutColors.push_back(0xFF * Color.r);
				OutColors.push_back(0xFF * Color.g);
				OutColors.push_back(0xFF * Color.b);
			}
			for (int64_t i = 0; i < IndexCounts[d]; i += 3)
			{
				const uint32_t* I = Indices + IndexBase + i;
				Triangles.emplace_back(Offset + I[0], Offset + I[1], Offset + I[2]);
			}
			Offset += (size_t)VertexCounts[d];
			IndexBase += (size_t)IndexCounts[d];
		}
		if (Format == 0) WriteSTL(std::string(Path), Vertices, OutNormals, Triangles);
		else WritePLY(std::string(Path), Vertices, OutColors, OutNormals, Triangles);
	}

	// SDFNode::RayMarch (sdf_evaluator.cpp:336-353) on the full tree.
	void ref_raymarch(void* Handle, int64_t Count, const float* Origins, const float* Dirs, int MaxIterations, float Epsilon,
		int Threads, uint8_t* Hit, float* Travel, float* Position)
	{
		SDFNodeShared Root = ((RefTree*)Handle)->Root;
		std::atomic<int64_t> Next(0);
		auto Thunk = [&]()
		{
			for (int64_t i = Next.fetch_add(64); i < Count; i = Next.fetch_add(64))
			{
				for (int64_t r = i; r < std::min<int64_t>(Count, i + 64); ++r)
				{
					RayHit H = Root->RayMarch(vec3(Origins[r * 3], Origins[r * 3 + 1], Origins[r * 3 + 2]),
						vec3(Dirs[r * 3], Dirs[r * 3 + 1], Dirs[r * 3 + 2]), MaxIterations, Epsilon);
					Hit[r] = H.Hit ? 1 : 0;
					Travel[r] = H.Travel;
					Position[r * 3 + 0] = H.Position.x;
					Position[r * 3 + 1] = H.Position.y;
					Position[r * 3 + 2] = H.Position.z;
				}
			}
		};
		if (Threads <= 0)
		{
			Pool(Thunk);
		}
		else
		{
			std::vector<std::thread> Workers;
			for (int t = 0; t < Threads; ++t) Workers.emplace_back(Thunk);
			for (auto& W : Workers) W.join();
		}
	}

	int ref_hardware_threads()
	{
		return (int)std::thread::hardware_concurrency();
	}
}
