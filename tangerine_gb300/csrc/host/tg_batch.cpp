#include "tg_batch.hpp"
#include "tg_surrogate.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <utility>

#define TG_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return _e; } while (0)

namespace tg
{
	Batch::Batch(std::vector<const Program*> programs, std::vector<GridSpec> grids, bool attributes)
		: Programs(std::move(programs)), Grids(std::move(grids)), Attributes(attributes)
	{
		Bricks.assign(Programs.size(), 7);
		Lanes.assign(Programs.size(), 2);
		cudaGetDevice(&DeviceId);
	}

	Batch::~Batch()
	{
		int prev = 0;
		const bool switched = cudaGetDevice(&prev) == cudaSuccess && prev != DeviceId && cudaSetDevice(DeviceId) == cudaSuccess;
		Release();
		if (switched) cudaSetDevice(prev);
	}

	void Batch::DropGraph()
	{
		if (GraphExec) cudaGraphExecDestroy(GraphExec);
		if (Graph) cudaGraphDestroy(Graph);
		GraphExec = nullptr;
		Graph = nullptr;
		if (Info.Graph == 1) Info.Graph = 0;      // capture again on the next run (a refusal stays)
	}

	void Batch::Release()
	{
		DropGraph();
		for (DeviceBuffer* b : { &Models, &BrickWord0, &CellBit0, &CellWords, &BrickBits, &BrickWordBase, &BrickList, &BrickTops, &CellBits,
			&CellWordBase, &ActiveCells, &Lattice, &Vertices, &Normals, &Colors, &Cubes, &FaceCounts, &FaceBase, &Faces,
			&VertexBase, &FaceBaseModel, &Counters, &ScanPartials, &Barrier, &Status, &Knobs })
			b->Release();
		if (HostCounters) cudaFreeHost(HostCounters);
		HostCounters = nullptr;
		std::lock_guard<std::mutex> l(CancelMutex);
		if (CancelHost) cudaFreeHost(CancelHost);
		CancelHost = CancelDevice = nullptr;
	}

	bool Batch::SetCancel(bool cancel)
	{
		std::lock_guard<std::mutex> l(CancelMutex);
		if (!CancelHost)
		{
			int dev = 0;
			if (cudaGetDevice(&dev) != cudaSuccess || dev != DeviceId) { cudaGetLastError(); return false; }
			if (cudaHostAlloc((void**)&CancelHost, sizeof(int), cudaHostAllocMapped) != cudaSuccess)
			{
				cudaGetLastError();
				CancelHost = nullptr;
				return false;
			}
			*CancelHost = 0;
			if (cudaHostGetDevicePointer((void**)&CancelDevice, CancelHost, 0) != cudaSuccess)
			{
				cudaGetLastError();
				cudaFreeHost(CancelHost);
				CancelHost = CancelDevice = nullptr;
				return false;
			}
		}
		*(volatile int*)CancelHost = cancel ? 1 : 0;
		return true;
	}

	void Batch::SetBarrierKnobs(uint64_t limit_ns, int late_block, uint64_t late_ns)
	{
		KnobHost[0] = limit_ns;
		KnobHost[1] = late_block >= 0 ? (uint64_t)late_block + 1 : 0;
		KnobHost[2] = late_ns;
	}

	void Batch::SetTuning(const std::vector<int>& bricks, const std::vector<int>& lanes)
	{
		for (size_t m = 0; m < Programs.size(); ++m)
		{
			if (m < bricks.size() && bricks[m] >= 1 && bricks[m] <= 32) Bricks[m] = bricks[m];
			if (m < lanes.size() && (lanes[m] == 1 || lanes[m] == 2 || lanes[m] == 4)) Lanes[m] = lanes[m];
		}
		Planned = false;
		DropGraph();
	}

	void Batch::SetFields(const std::vector<const FieldNet*>& fields, bool refine)
	{
		Fields = fields;
		Fields.resize(Programs.size(), nullptr);
		FieldRefine = refine;
		Planned = false;
		DropGraph();
	}

	cudaError_t Batch::Plan(cudaStream_t s)
	{
		const int n = (int)Programs.size();
		std::vector<BatchModel> models((size_t)n);
		std::vector<int64_t> bw0((size_t)n), cw((size_t)n), t0((size_t)n);
		int64_t tiles = 0;
		std::vector<uint64_t> cb0((size_t)n);
		HasPaint.assign((size_t)n, 0);
		int64_t bword = 0, cword = 0, lat = 0, bricks = 0, samples = 0;
		double capV = 0.0;
		MaxStack = 1;
		for (int m = 0; m < n; ++m)
		{
			const GridSpec& g = Grids[m];
			const int B = Bricks[m];
			BatchModel& bm = models[m];
			bm.Prog = Programs[m]->View;
			bm.Grid = g;
			bm.B = B;
			bm.NBX = (g.NX - 1 + B - 1) / B;
			bm.NBY = (g.NY - 1 + B - 1) / B;
			bm.NBZ = (g.NZ - 1 + B - 1) / B;
			bm.Lanes = Lanes[m];
			bm.HasPaint = HasPaint[m] = Programs[m]->Host.Header.HasPaint ? 1 : 0;
			bm.Bricks = (int64_t)bm.NBX * bm.NBY * bm.NBZ;
			bm.Lattice = lat;
			bm.BrickWord0 = bw0[m] = bword;
			bm.CellWord0 = cword;
			bm.Cull = (m < (int)Fields.size() && Fields[m]) ? (FieldRefine ? 2 : 1) : 0;
			t0[m] = tiles;
			tiles += (int64_t)((bm.NBX + 7) / 8) * ((bm.NBY + 3) / 4) * bm.NBZ;
			const int64_t sx = g.NX - 1, sy = g.NY - 1, sz = g.NZ - 1;
			cw[m] = (sx * sy * sz + 31) / 32;
			cb0[m] = (uint64_t)cword * 32u;
			bword += (bm.Bricks + 31) / 32;
			cword += cw[m];
			lat += (int64_t)g.NX * g.NY * g.NZ;
			bricks += bm.Bricks;
			samples += (int64_t)g.NX * g.NY * g.NZ;
			capV += 10.0 * (double)std::max({ sx * sy, sy * sz, sx * sz }) + 4096.0;
			MaxStack = std::max(MaxStack, bm.Prog.MaxStack);
		}
		BrickWordHost = bw0;
		if ((double)bword * 32.0 >= 4294967296.0) { SetError("batch too large: more than 2^32 bricks"); return cudaErrorInvalidValue; }
		CapVertices = ReqVertices ? ReqVertices : (uint32_t)std::min(capV, 4.0e9 / 2.5);
		CapFaces = ReqFaces ? ReqFaces : (uint32_t)std::min(2.5 * (double)CapVertices, 4.0e9);
		Info.Models = n;
		Info.Bricks = bricks;
		Info.Samples = samples;

		TG_TRY(Models.Reserve(sizeof(BatchModel) * (size_t)n));
		TG_TRY(BrickWord0.Reserve(8 * (size_t)n));
		TG_TRY(CellBit0.Reserve(8 * (size_t)n));
		TG_TRY(CellWords.Reserve(8 * (size_t)n));
		TG_TRY(Tile0.Reserve(8 * (size_t)n));
		TG_TRY(BrickBits.Reserve(4 * (size_t)bword));
		TG_TRY(BrickWordBase.Reserve(4 * (size_t)bword));
		TG_TRY(BrickList.Reserve(4 * (size_t)bword * 32));
		TG_TRY(BrickTops.Reserve(4 * (size_t)bword * 32));
		TG_TRY(CellBits.Reserve(4 * (size_t)cword));
		TG_TRY(CellWordBase.Reserve(4 * (size_t)cword));
		TG_TRY(Lattice.Reserve(4 * (size_t)lat));
		TG_TRY(VertexBase.Reserve(4 * ((size_t)n + 1)));
		TG_TRY(FaceBaseModel.Reserve(4 * ((size_t)n + 1)));
		TG_TRY(Counters.Reserve(16 * 4));
		TG_TRY(Barrier.Reserve(8));
		TG_TRY(Status.Reserve(4));
		TG_TRY(Knobs.Reserve(4 * sizeof(uint64_t)));
		if (!CancelHost && !SetCancel(false)) { SetError("cannot map the batch's cancel flag"); return cudaErrorMemoryAllocation; }
		if (!HostCounters) TG_TRY(cudaMallocHost(&HostCounters, 8 * sizeof(uint32_t)));
		TG_TRY(BatchMaxBlocks(MaxStack, &Blocks));
		if (Blocks <= 0) { SetError("the batch kernel does not fit on this device"); return cudaErrorInvalidConfiguration; }
		TG_TRY(ScanPartials.Reserve(4 * ((size_t)Blocks + 1)));
		TG_TRY(cudaMemcpyAsync(Models.Ptr, models.data(), sizeof(BatchModel) * (size_t)n, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaMemcpyAsync(BrickWord0.Ptr, bw0.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaMemcpyAsync(CellBit0.Ptr, cb0.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaMemcpyAsync(CellWords.Ptr, cw.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaMemcpyAsync(Tile0.Ptr, t0.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaStreamSynchronize(s));

		State = BatchState{};
		State.Models = Models.As<BatchModel>();
		State.Count = n;
		State.Attributes = Attributes ? 1 : 0;
		State.BrickWord0 = BrickWord0.As<int64_t>();
		State.CellBit0 = CellBit0.As<uint64_t>();
		State.CellWords = CellWords.As<int64_t>();
		State.BrickWordsTotal = bword;
		State.Tile0 = Tile0.As<int64_t>();
		State.TilesTotal = tiles;
		State.CellWordsTotal = cword;
		State.BrickBits = BrickBits.As<uint32_t>();
		State.BrickWordBase = BrickWordBase.As<uint32_t>();
		State.BrickList = BrickList.As<uint32_t>();
		State.BrickTops = BrickTops.As<uint32_t>();
		State.CellBits = CellBits.As<uint32_t>();
		State.CellWordBase = CellWordBase.As<uint32_t>();
		State.Lattice = Lattice.As<float>();
		State.VertexBase = VertexBase.As<uint32_t>();
		State.FaceBaseModel = FaceBaseModel.As<uint32_t>();
		State.Counters = Counters.As<uint32_t>();
		State.ScanPartials = ScanPartials.As<uint32_t>();
		State.Barrier = Barrier.As<unsigned>();
		State.Status = Status.As<int>();
		State.Cancel = CancelDevice;
		State.Knobs = Knobs.As<uint64_t>();
		Planned = true;
		return cudaSuccess;
	}

	cudaError_t Batch::Launch(cudaStream_t s)
	{
		// Output buffers sized by the current capacities.
		TG_TRY(ActiveCells.Reserve(8 * (size_t)CapVertices));
		TG_TRY(Vertices.Reserve(12 * (size_t)CapVertices));
		TG_TRY(Cubes.Reserve(4 * (size_t)CapVertices));
		TG_TRY(FaceCounts.Reserve(4 * (size_t)CapVertices));
		TG_TRY(FaceBase.Reserve(4 * (size_t)CapVertices));
		TG_TRY(Faces.Reserve(12 * (size_t)CapFaces));
		if (Attributes)
		{
			TG_TRY(Normals.Reserve(12 * (size_t)CapVertices));
			TG_TRY(Colors.Reserve(3 * (size_t)CapVertices));
		}
		State.CapVertices = CapVertices;
		State.CapFaces = CapFaces;
		State.ActiveCells = ActiveCells.As<uint64_t>();
		State.Vertices = Vertices.As<float>();
		State.Cubes = Cubes.As<uint32_t>();
		State.FaceCounts = FaceCounts.As<uint32_t>();
		State.FaceBase = FaceBase.As<uint32_t>();
		State.Faces = Faces.As<uint32_t>();
		State.Normals = Normals.As<float>();
		State.Colors = Colors.As<uint8_t>();

		auto enqueue = [&]() -> cudaError_t {
			TG_TRY(cudaMemsetAsync(Counters.Ptr, 0, 16 * 4, s));
			TG_TRY(cudaMemsetAsync(Barrier.Ptr, 0, 8, s));
			TG_TRY(cudaMemsetAsync(Status.Ptr, 0, 4, s));
			// Models with a learned bound: its brick bits first, into the model's words.
			for (size_t m = 0; m < Fields.size() && m < Programs.size(); ++m)
			{
				const FieldNet* f = Fields[m];
				if (!f) continue;
				const GridSpec& g = Grids[m];
				const int B = Bricks[m];
				const float radius = 0.8660254f * (float)B * std::max(g.DX, std::max(g.DY, g.DZ));
				TG_TRY(LaunchFieldClassifyBricks(Programs[m]->View, g, B, f->Grid, f->TablePtr(), f->ImagePtr(), f->MarginFor(radius),
					BrickBits.As<uint32_t>() + BrickWordHost[m], f->StatusPtr(), s));
			}
			return LaunchBatchExport(State, Blocks, MaxStack, s);
		};
		if (!GraphExec && !Info.Graph)
		{
			// Capture the whole batch (resets + the cooperative launch) once; replay it after.
			if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
			{
				const cudaError_t e = enqueue();
				cudaGraph_t g = nullptr;
				const cudaError_t ce = cudaStreamEndCapture(s, &g);
				if (e == cudaSuccess && ce == cudaSuccess && g && cudaGraphInstantiate(&GraphExec, g, 0) == cudaSuccess)
				{
					Graph = g;
					Info.Graph = 1;
				}
				else
				{
					if (g) cudaGraphDestroy(g);
					GraphExec = nullptr;
					cudaGetLastError();
					Info.Graph = -1;      // capture refused: launch directly from now on
				}
			}
			else
			{
				cudaGetLastError();
				Info.Graph = -1;
			}
		}
		if (GraphExec) return cudaGraphLaunch(GraphExec, s);
		return enqueue();
	}

	cudaError_t Batch::Run(cudaStream_t s)
	{
		if (!Planned) TG_TRY(Plan(s));
		const int n = (int)Programs.size();
		Info.Reruns = 0;
		LastStatus = 0;
		for (int attempt = 0; attempt < 3; ++attempt)
		{
			TG_TRY(cudaMemcpyAsync(Knobs.Ptr, KnobHost, sizeof KnobHost, cudaMemcpyHostToDevice, s));
			TG_TRY(Launch(s));
			TG_TRY(cudaMemcpyAsync(HostCounters, Counters.Ptr, 5 * 4, cudaMemcpyDeviceToHost, s));
			TG_TRY(cudaMemcpyAsync(HostCounters + 5, Status.Ptr, 4, cudaMemcpyDeviceToHost, s));
			TG_TRY(cudaStreamSynchronize(s));
			if (HostCounters[5] != 0)
			{
				LastStatus = (int)HostCounters[5];
				if (LastStatus == 3)
				{
					SetCancel(false);
					SetError("the batch run was cancelled");
					return cudaSuccess;
				}
				SetError("the batch kernel's grid barrier timed out");
				return cudaErrorLaunchTimeout;
			}
			for (const FieldNet* f : Fields)
				if (f) TG_TRY(const_cast<FieldNet*>(f)->CheckStatus(s));
			const uint32_t overflow = HostCounters[4];
			if (!overflow) break;
			// Outputs did not fit: grow to the counts this run found and run again.
			const double v = (double)HostCounters[2];
			const double f = (overflow & 1u) ? 2.5 * v : (double)HostCounters[3];
			CapVertices = (uint32_t)std::min(std::max((double)CapVertices, 1.1 * v + 4096.0), 4.0e9 / 2.5);
			CapFaces = (uint32_t)std::min(std::max((double)CapFaces, 1.1 * f + 4096.0), 4.0e9);
			DropGraph();
			++Info.Reruns;
			if (attempt == 2) { SetError("batch outputs did not fit after growing twice"); return cudaErrorMemoryAllocation; }
		}
		Info.BricksEvaluated = HostCounters[0];
		Info.Vertices = HostCounters[2];
		Info.Faces = HostCounters[3];
		Info.Blocks = Blocks;
		HostVertexBase.resize((size_t)n + 1);
		HostFaceBase.resize((size_t)n + 1);
		TG_TRY(cudaMemcpyAsync(HostVertexBase.data(), VertexBase.Ptr, 4 * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaMemcpyAsync(HostFaceBase.data(), FaceBaseModel.Ptr, 4 * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		int64_t bytes = 0;
		for (const DeviceBuffer* b : { &Models, &BrickWord0, &CellBit0, &CellWords, &BrickBits, &BrickWordBase, &BrickList, &BrickTops, &CellBits,
			&CellWordBase, &ActiveCells, &Lattice, &Vertices, &Normals, &Colors, &Cubes, &FaceCounts, &FaceBase, &Faces,
			&VertexBase, &FaceBaseModel, &Counters, &ScanPartials, &Barrier, &Status, &Knobs })
			bytes += (int64_t)b->Bytes;
		Info.DeviceBytes = bytes;
		return cudaSuccess;
	}

	void Batch::Reserve(uint32_t vertices, uint32_t faces)
	{
		ReqVertices = CapVertices = std::max<uint32_t>(vertices, 1);
		ReqFaces = CapFaces = std::max<uint32_t>(faces, 1);
		DropGraph();
	}

	void Batch::MeshOf(int m, DeviceMesh& out) const
	{
		out = DeviceMesh();
		if (m < 0 || (size_t)m + 1 >= HostVertexBase.size()) return;
		const uint32_t v0 = HostVertexBase[m], v1 = HostVertexBase[m + 1];
		const uint32_t f0 = HostFaceBase[m], f1 = HostFaceBase[m + 1];
		out.VertexCount = v1 - v0;
		out.FaceCount = f1 - f0;
		out.Vertices = Vertices.As<float>() + (size_t)v0 * 3;
		out.Cubes = Cubes.As<uint32_t>() + v0;
		out.Faces = Faces.As<uint32_t>() + (size_t)f0 * 3;
		if (Attributes)
		{
			out.Normals = Normals.As<float>() + (size_t)v0 * 3;
			out.Colors = HasPaint[m] ? Colors.As<uint8_t>() + (size_t)v0 * 3 : nullptr;
		}
	}

	cudaError_t Batch::Autotune(cudaStream_t s)
	{
		const auto t0 = std::chrono::steady_clock::now();
		Engine& eng = Engine::Get();
		// Class: largest lattice extent and log2 of the distance program's size.
		std::map<std::pair<int, int>, std::vector<int>> classes;
		for (size_t m = 0; m < Programs.size(); ++m)
		{
			const GridSpec& g = Grids[m];
			const int extent = std::max({ g.NX, g.NY, g.NZ });
			const int quads = std::max<int>(1, (int)Programs[m]->Host.Header.CodeQuads);
			classes[{ extent, (int)std::log2((double)quads) }].push_back((int)m);
		}
		const int brickChoices[] = { 4, 7, 11, 15 };
		const int laneChoices[] = { 1, 2, 4 };
		for (auto& kv : classes)
		{
			const int rep = kv.second.front();
			double best = 1e30;
			int bestB = 7, bestL = 2;
			for (int B : brickChoices)
			{
				for (int L : laneChoices)
				{
					ExportOptions opt;
					opt.Attributes = Attributes;
					opt.BrickSize = B;
					opt.Lanes = L;
					double fastest = 1e30;
					for (int rep_i = 0; rep_i < 3; ++rep_i)
					{
						DeviceMesh dm;
						const auto a = std::chrono::steady_clock::now();
						TG_TRY(eng.Export(*Programs[rep], Grids[rep], opt, dm, s));
						const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
						if (rep_i > 0) fastest = std::min(fastest, dt);
					}
					if (fastest < best) { best = fastest; bestB = B; bestL = L; }
				}
			}
			for (int m : kv.second) { Bricks[m] = bestB; Lanes[m] = bestL; }
		}
		Planned = false;
		DropGraph();
		Info.AutotuneSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
		return cudaSuccess;
	}
}
