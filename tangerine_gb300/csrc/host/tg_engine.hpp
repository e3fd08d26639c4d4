// Per-process GPU engine: device buffers reused across calls, the export pipeline and an
// optional per-kernel profiler.
#pragma once

#include <atomic>
#include <cstdint>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "tg_layout.hpp"
#include "tg_octree.hpp"
#include "../kernels/tg_kernels.hpp"

namespace tg
{
	class FieldNet;

	// A grow-only device allocation.
	struct DeviceBuffer
	{
		void* Ptr = nullptr;
		size_t Bytes = 0;
		cudaError_t Reserve(size_t bytes);
		void Release();
		template<typename T> T* As() const { return static_cast<T*>(Ptr); }
	};

	struct Program
	{
		CompiledTree Host;
		void* Device = nullptr;
		DeviceProgram View{};
		int DeviceId = 0;
		bool OwnsDevice = true;      // false: the bytes live in the engine's scratch program buffer
		~Program();
	};

	struct DeviceMesh
	{
		uint64_t VertexCount = 0;
		uint64_t FaceCount = 0;
		float* Vertices = nullptr;
		float* Normals = nullptr;
		uint8_t* Colors = nullptr;
		uint32_t* Faces = nullptr;
		uint32_t* Cubes = nullptr;
	};

	// Host blocks an export fills itself (allocated from the pinned pool once the counts are
	// known): the vertices, cubes and faces are copied on a second stream while the normals
	// and colours are still being computed.
	struct HostMeshOut
	{
		uint64_t VertexCount = 0, FaceCount = 0;
		float* Vertices = nullptr;
		float* Normals = nullptr;
		uint8_t* Colors = nullptr;
		uint32_t* Faces = nullptr;
		uint32_t* Cubes = nullptr;
		bool OutOfMemory = false;
	};
	void FreeHostMesh(HostMeshOut& m);

	struct ExportOptions
	{
		bool Attributes = true;     // gradient normals and colours
		bool Dense = false;         // evaluate every lattice point (no brick culling)
		int BrickSize = 7;          // cells per brick edge when culling (1..32)
		int Lanes = 2;              // lattice points per thread sharing one pass over records
		bool Staged = false;        // brick evaluation reads single-cell bricks' programs from shared memory
		const FieldNet* Field = nullptr;    // learned bound for the brick test (else exact)
		bool Refine = true;                 // with Field: network-kept bricks also take the exact test
		// The exact brick test already ran on the root cell's program (Engine::PreClassify,
		// same grid and brick size, same stream): the export lists its bricks and descends
		// them instead of classifying.
		bool PreClassified = false;
		// Host work to run while the export waits for its first count read-back (an error
		// from it ends the export), and RestageCode: the program's code region is copied to
		// the device again from the engine's staging buffer once the kernels that read
		// distance programs are done, and the vertex attribute pass waits for that copy --
		// for a program uploaded with UploadScratch whose surface programs that host work
		// wrote into the staged image (FinishSurfaces).
		std::function<cudaError_t()> WhileWaiting;
		bool RestageCode = false;
		HostMeshOut* Host = nullptr;        // also copy the mesh to host memory (see HostMeshOut)
		// Host-side control of an asynchronous export (MeshExport): when *Active turns false
		// the export stops at its next synchronisation point, sets *Cancelled and returns an
		// empty mesh; *Progress receives the share of its phases done (0..1).
		const std::atomic<bool>* Active = nullptr;
		bool* Cancelled = nullptr;
		std::atomic<float>* Progress = nullptr;
		// The asynchronous export's stage word (ExportProgress::Stage): the point-cloud
		// export stores 2 when its voxel search ends and skips the refinement when the word
		// has moved past 2 by then (CancelExport(false) during the refinement stage).
		std::atomic<int>* Stage = nullptr;
	};

	// Sodapop's meshing job output (device pointers into the engine's buffers, valid until
	// the next call on the engine).
	struct SodapopMesh
	{
		uint64_t VertexCount = 0;
		uint64_t FaceCount = 0;
		float* Positions = nullptr;   // 3 per vertex
		float* Normals = nullptr;     // 3 per vertex
		float* Colors = nullptr;      // 4 per vertex
		uint32_t* Faces = nullptr;    // 3 per face
		uint32_t* Cells = nullptr;    // cell number per vertex
		SodapopGrid Grid{};
	};

	// NaiveSurfaceNetsScratch's lattice (sodapop.cpp:150-177) for a program compiled with
	// OctreeKind::Meshing at `density` samples per unit, and the integer boxes of its
	// leaves' point-cache spans (sodapop.cpp:622-644).  False (with a reason) when the
	// lattice is outside what the kernels index.
	bool SodapopPlan(const CompiledTree& t, float density, SodapopGrid& g, std::vector<int64_t>& boxes, std::string& error);

	// PointCloudExportThread's lattice (export.cpp:384-400) for (min, max, step); false
	// when it is empty or beyond the reference's int cell numbers.
	bool CloudPlan(const float lo[3], const float hi[3], const float step[3], CloudSpec& s, std::string& error);
	// VoxExport's lattice and radius (magica.cpp:29-40) over `bounds` at grid_size.
	bool VoxPlan(const AABB& bounds, float grid_size, VoxSpec& s, std::string& error);
	// VoxWriter::SaveToFile (voxwriter/VoxWriter.cpp:560-660) for voxels (x, y, z, colour
	// index) added in the given order to a writer whose cube limits are `size`.
	bool WriteVoxFile(const std::string& path, const int32_t size[3], const int32_t* xyzc, size_t count);

	class Engine
	{
	public:
		static Engine& Get();

		cudaStream_t DefaultStream();
		cudaError_t Upload(Program& p);
		// Upload into the engine's reusable program buffer, asynchronously on `s` (for a
		// program used by one call only, such as tg_export_tree's).
		cudaError_t UploadScratch(Program& p, cudaStream_t s);
		// The code image UploadScratch last staged for `p` (pinned host memory, quad 0
		// first), and a copy of that code region to the device again on `s`.
		float* StagedCode(const Program& p);
		cudaError_t RestageCode(const Program& p, cudaStream_t s);
		cudaError_t EvalGrid(const Program& p, const GridSpec& g, float* device_out, cudaStream_t s);
		cudaError_t EvalPoints(const Program& p, const float* host_points, int64_t n, float* host_out, cudaStream_t s);
		cudaError_t Export(const Program& p, const GridSpec& g, const ExportOptions& opt, DeviceMesh& out, cudaStream_t s);
		// The exact brick test of a culled export on the root cell's program alone (the
		// root's own sphere holds every ball it decides, so it is the test's holder of last
		// resort), launched on `s` while the host is still building the octree below the
		// root.  An export of the same grid and brick size on `s` with PreClassified set
		// takes its brick bits; any other engine call in between voids them.
		cudaError_t PreClassify(const RootProgram& root, const GridSpec& g, int brick_size, cudaStream_t s);
		int64_t LastActiveBricks() const { return ActiveBricks; }
		// The kept bricks of the last culled export (brick index order), copied to host.
		cudaError_t LastBrickList(std::vector<uint32_t>& out, int& brick_size);
		int64_t LastBricks() const { return Bricks; }
		cudaError_t FaceNormals(const Program& p, const float* host_vertices, uint64_t vertex_count, const uint32_t* host_faces,
			uint64_t face_count, float* host_normals, cudaStream_t s);
		cudaError_t RayMarch(const Program& p, const float* origins, const float* dirs, int64_t n, int iterations, float epsilon,
			uint8_t* hit, float* travel, float* position, cudaStream_t s, const RayFrame* frame = nullptr);
		// SDFNode::Eval (gradient = false, 1 float per point) or SDFNode::Gradient (3) on the
		// whole tree at host points.
		cudaError_t PointQuery(const Program& p, const float* points, int64_t n, bool gradient, float* out, cudaStream_t s);
		cudaError_t Render(const Program& p, const CameraBasis* cams, int count, int width, int height, int steps, float epsilon,
			bool exact, float* depth, float* normals, uint8_t* colors, bool out_is_device, cudaStream_t s, const FieldNet* field = nullptr);
		// Sodapop's meshing job (MeshingJob::NaiveSurfaceNets) for a program compiled with
		// OctreeKind::Meshing, planned by SodapopPlan.
		cudaError_t Sodapop(const Program& p, const SodapopGrid& g, const std::vector<int64_t>& boxes, SodapopMesh& out,
			cudaStream_t s);
		// PointCloudExportThread on the GPU: the kept voxel centres (cell order), refined,
		// with gradient normals and colours when `attributes`; Cubes holds each point's
		// voxel number, Faces nothing.
		cudaError_t PointCloud(const Program& p, const CloudSpec& s, int refine, bool attributes, DeviceMesh& out, cudaStream_t st,
			const ExportOptions* control = nullptr);
		// VoxExport's voxel test on the GPU: the kept voxel numbers in order, to the host.
		cudaError_t Voxels(const Program& p, const VoxSpec& s, std::vector<uint32_t>& cells, cudaStream_t st);
		// Network iterations and exact steps of the last network-stepped render.
		uint64_t LastNetworkSteps = 0, LastExactSteps = 0;
		DeviceBuffer& Lattice() { return LatticeBuf; }

		// Profiling of kernel launches (CUDA events on the launching stream).
		void SetProfiling(bool on);
		bool ReadProfile(const std::string& name, double& ms, int64_t& launches);
		void ResetProfile();
		std::mutex Mutex;   // engine calls are serialised

	private:
		Engine() = default;
		struct Mark { std::string Name; cudaEvent_t Start, Stop; };
		struct Total { std::string Name; double Ms; int64_t Launches; };
		void Begin(const char* name, cudaStream_t s);
		void End(cudaStream_t s);
		void Collect();
		bool Profiling = false;
		std::vector<Mark> Pending;
		std::vector<Total> Totals;

		cudaStream_t Stream = nullptr;
		cudaStream_t CopyStream = nullptr;          // early device-to-host copies of an export
		cudaEvent_t MeshReady = nullptr;
		cudaEvent_t CodeReady = nullptr;            // RestageCode's copy of an export is done
		DeviceBuffer LatticeBuf, Words, WordBase, Scratch, Counts, Vertices, Cubes, FaceCounts, FaceBase, Faces, Normals, Colors;
		DeviceBuffer Points, PointOut, BrickBits, BrickList, BrickTops, ClassCounts, ProgramScratch, ActiveCells;
		DeviceBuffer RayIn, RayOut, Cameras, Image, RenderCounters;
		DeviceBuffer SodaBoxes, SodaCache, SodaColors;
		void* Staging = nullptr;
		size_t StagingBytes = 0;
		// PreClassify's one-cell program: pinned staging, its device copy, the event after
		// the copy (the staging is rewritten only once the last copy out of it is done),
		// and the grid and brick size whose bits it left in BrickBits.
		DeviceBuffer RootScratch;
		void* RootStaging = nullptr;
		size_t RootStagingBytes = 0;
		cudaEvent_t RootCopied = nullptr;
		bool RootCopyPending = false;
		bool PreValid = false;
		GridSpec PreGrid{};
		int PreBrickSize = 0;
		uint32_t* HostCounts = nullptr;
		int SmCount = 0;
		int64_t ActiveBricks = 0, Bricks = 0;
		int LastBrickSize = 0;
	};

	// Pinned host blocks handed out as mesh outputs and taken back by tg_mesh_free, so the
	// device-to-host copies run at full link speed without pinning memory on every call.
	class HostPool
	{
	public:
		static HostPool& Get();
		void* Take(size_t bytes);            // nullptr when pinned memory is unavailable
		bool Give(void* p);                  // false: p is not from this pool
	private:
		std::mutex Mutex;
		std::vector<std::pair<void*, size_t>> Free;
		std::vector<std::pair<void*, size_t>> Used;
	};

	struct ExportTiming
	{
		double CompileSeconds = 0, UploadSeconds = 0, GpuSeconds = 0, CopySeconds = 0;
	};
	ExportTiming& LastTiming();

	std::string& LastError();
	void SetError(const std::string& msg);
}

// The opaque handle of the C ABI (include/tangerine_gb300.h) is a compiled program.
struct tg_program : public tg::Program {};
