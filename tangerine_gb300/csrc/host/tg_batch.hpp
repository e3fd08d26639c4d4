// Many compiled trees exported together by one persistent cooperative launch
// (kernels/tg_batch.cu), replayed from a CUDA graph, with per-model brick size and lattice
// points per thread chosen by an autotuner.
#pragma once

#include <cstdint>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "tg_engine.hpp"

namespace tg
{
	struct BatchInfo
	{
		int64_t Models = 0, Samples = 0, Bricks = 0, BricksEvaluated = 0, Vertices = 0, Faces = 0;
		int Graph = 0, Blocks = 0, Reruns = 0;
		double AutotuneSeconds = 0;
		int64_t DeviceBytes = 0;
	};

	class Batch
	{
	public:
		Batch(std::vector<const Program*> programs, std::vector<GridSpec> grids, bool attributes);
		~Batch();

		// Per-model brick edge (cells) and lattice points per thread; invalidates the plan.
		void SetTuning(const std::vector<int>& bricks, const std::vector<int>& lanes);
		// Times single-model exports of one representative per (resolution, program size)
		// class for every candidate (brick edge, lanes) and gives each class its fastest.
		cudaError_t Autotune(cudaStream_t s);
		cudaError_t Run(cudaStream_t s);
		// Learned distance bounds per model (null: exact test), which cull the model's bricks
		// before the launch; with `refine` the bricks a bound keeps also take the exact test.
		// The nets must outlive the batch's runs.  Invalidates the plan.
		void SetFields(const std::vector<const FieldNet*>& fields, bool refine);
		// Output capacities (vertices, faces) for the next run; a run that finds more grows
		// them and runs again.
		void Reserve(uint32_t vertices, uint32_t faces);
		// Model m's slice of the outputs (device pointers; faces hold the model's own
		// vertex numbers).  Valid until the next Run.
		void MeshOf(int m, DeviceMesh& out) const;
		// Sets (or withdraws) the cancel flag the running kernel polls at its grid barriers;
		// callable from any thread.  False when the flag could not be allocated.
		bool SetCancel(bool cancel);
		// Grid-barrier test hook: time limit (0: default) and one block started late.
		void SetBarrierKnobs(uint64_t limit_ns, int late_block, uint64_t late_ns);
		// Outcome of the last Run's kernel: 0, 2 (a barrier wait ran out) or 3 (cancelled).
		int LastStatus = 0;

		std::vector<int> Bricks, Lanes;
		BatchInfo Info;

	private:
		cudaError_t Plan(cudaStream_t s);
		cudaError_t Launch(cudaStream_t s);
		void DropGraph();
		void Release();

		std::vector<const Program*> Programs;
		std::vector<GridSpec> Grids;
		std::vector<const FieldNet*> Fields;
		bool FieldRefine = true;
		bool Attributes;
		bool Planned = false;
		int MaxStack = 1, Blocks = 0;
		uint32_t CapVertices = 0, CapFaces = 0;
		uint32_t ReqVertices = 0, ReqFaces = 0;     // capacities asked for by Reserve (0: estimate)
		BatchState State{};
		DeviceBuffer Models, BrickWord0, Tile0, CellBit0, CellWords, BrickBits, BrickWordBase, BrickList, BrickTops, CellBits, CellWordBase,
			ActiveCells, Lattice, Vertices, Normals, Colors, Cubes, FaceCounts, FaceBase, Faces, VertexBase, FaceBaseModel,
			Counters, ScanPartials, Barrier, Status, Knobs;
		int* CancelHost = nullptr;                 // host-mapped page-locked flag
		int* CancelDevice = nullptr;               // its device address
		uint64_t KnobHost[4] = {};
		std::vector<uint32_t> HostVertexBase, HostFaceBase;
		std::vector<int64_t> BrickWordHost;        // per model: first word of its brick bits
		std::vector<int> HasPaint;
		uint32_t* HostCounters = nullptr;
		cudaGraph_t Graph = nullptr;
		cudaGraphExec_t GraphExec = nullptr;
		int DeviceId = 0;
		std::mutex CancelMutex;
	};
}

struct tg_batch : public tg::Batch
{
	using tg::Batch::Batch;
};
