// GPU engine: device buffers, the export pipeline and the kernel profiler.
#include "tg_engine.hpp"
#include "tg_surrogate.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>

namespace tg
{
	std::string& LastError()
	{
		static thread_local std::string msg;
		return msg;
	}

	void SetError(const std::string& msg) { LastError() = msg; }

	ExportTiming& LastTiming()
	{
		static thread_local ExportTiming t;
		return t;
	}

	HostPool& HostPool::Get()
	{
		static HostPool* pool = new HostPool();
		return *pool;
	}

	void* HostPool::Take(size_t bytes)
	{
		std::lock_guard<std::mutex> lock(Mutex);
		size_t best = (size_t)-1;
		for (size_t i = 0; i < Free.size(); ++i)
		{
			if (Free[i].second >= bytes && (best == (size_t)-1 || Free[i].second < Free[best].second)) best = i;
		}
		if (best != (size_t)-1)
		{
			auto blk = Free[best];
			Free.erase(Free.begin() + (long)best);
			Used.push_back(blk);
			return blk.first;
		}
		void* p = nullptr;
		const size_t want = bytes < 4096 ? 4096 : bytes + bytes / 8;
		if (cudaMallocHost(&p, want) != cudaSuccess) { cudaGetLastError(); return nullptr; }
		Used.push_back({ p, want });
		return p;
	}

	bool HostPool::Give(void* p)
	{
		if (!p) return true;
		std::lock_guard<std::mutex> lock(Mutex);
		for (size_t i = 0; i < Used.size(); ++i)
		{
			if (Used[i].first == p)
			{
				Free.push_back(Used[i]);
				Used.erase(Used.begin() + (long)i);
				return true;
			}
		}
		return false;
	}

	cudaError_t DeviceBuffer::Reserve(size_t bytes)
	{
		if (bytes <= Bytes && Ptr) return cudaSuccess;
		Release();
		size_t want = bytes < 256 ? 256 : bytes;
		cudaError_t e = cudaMalloc(&Ptr, want);
		if (e != cudaSuccess) { Ptr = nullptr; Bytes = 0; return e; }
		Bytes = want;
		return cudaSuccess;
	}

	void DeviceBuffer::Release()
	{
		if (Ptr) cudaFree(Ptr);
		Ptr = nullptr;
		Bytes = 0;
	}

	Program::~Program()
	{
		if (Device && OwnsDevice) cudaFree(Device);
	}

	Engine& Engine::Get()
	{
		static Engine* engine = new Engine();   // lives until exit; device memory goes with the context
		return *engine;
	}

	cudaStream_t Engine::DefaultStream()
	{
		if (!Stream) cudaStreamCreateWithFlags(&Stream, cudaStreamNonBlocking);
		return Stream;
	}

	namespace
	{
		inline size_t AlignUp(size_t v, size_t a) { return (v + a - 1) / a * a; }
	}

	namespace
	{
		struct ProgramLayout
		{
			size_t NodeBytes, CodeOff, CodeBytes, ColorOff, RgbOff, Total;
		};

		// Nodes, code quads, colour bytes, material RGB: each part 256-byte aligned.
		ProgramLayout LayoutOf(const Program& p)
		{
			ProgramLayout l;
			l.NodeBytes = p.Host.Nodes.size() * sizeof(OctNode);
			l.CodeOff = AlignUp(l.NodeBytes, 256);
			l.CodeBytes = p.Host.CodeFloats * sizeof(float);
			l.ColorOff = AlignUp(l.CodeOff + l.CodeBytes, 256);
			l.RgbOff = AlignUp(l.ColorOff + (p.Host.Colors.size() ? p.Host.Colors.size() : 4), 256);
			l.Total = l.RgbOff + (p.Host.MaterialRgb.size() ? p.Host.MaterialRgb.size() * sizeof(float) : 16);
			return l;
		}

		void Pack(const Program& p, const ProgramLayout& l, uint8_t* dst)
		{
			std::memcpy(dst, p.Host.Nodes.data(), l.NodeBytes);
			p.Host.CopyCode(reinterpret_cast<float*>(dst + l.CodeOff));
			if (!p.Host.Colors.empty()) std::memcpy(dst + l.ColorOff, p.Host.Colors.data(), p.Host.Colors.size());
			if (!p.Host.MaterialRgb.empty())
				std::memcpy(dst + l.RgbOff, p.Host.MaterialRgb.data(), p.Host.MaterialRgb.size() * sizeof(float));
		}

		void Bind(Program& p, const ProgramLayout& l, void* device)
		{
			uint8_t* base = static_cast<uint8_t*>(device);
			p.View.Nodes = reinterpret_cast<const OctNode*>(base);
			p.View.Code = reinterpret_cast<const float4*>(base + l.CodeOff);
			p.View.Colors = reinterpret_cast<const uchar4*>(base + l.ColorOff);
			p.View.MaterialRgb = reinterpret_cast<const float4*>(base + l.RgbOff);
			p.View.MaxStack = p.Host.Header.MaxStack;
			p.View.FullSurfaceCode = p.Host.Header.FullSurfaceCode;
			p.View.Lipschitz = p.Host.Header.Lipschitz;
		}
	}

	cudaError_t Engine::UploadScratch(Program& p, cudaStream_t s)
	{
		const ProgramLayout l = LayoutOf(p);
		cudaError_t e = cudaGetDevice(&p.DeviceId);
		if (e != cudaSuccess) return e;
		e = ProgramScratch.Reserve(l.Total);
		if (e != cudaSuccess) return e;
		if (StagingBytes < l.Total)
		{
			if (Staging) cudaFreeHost(Staging);
			Staging = nullptr;
			StagingBytes = 0;
			e = cudaMallocHost(&Staging, l.Total + l.Total / 4);
			if (e != cudaSuccess) { Staging = nullptr; return e; }
			StagingBytes = l.Total + l.Total / 4;
		}
		// The previous call's copy out of the staging buffer has finished: every export
		// synchronises its stream before returning.
		Pack(p, l, static_cast<uint8_t*>(Staging));
		e = cudaMemcpyAsync(ProgramScratch.Ptr, Staging, l.Total, cudaMemcpyHostToDevice, s);
		if (e != cudaSuccess) return e;
		p.Device = ProgramScratch.Ptr;
		p.OwnsDevice = false;
		Bind(p, l, p.Device);
		return cudaSuccess;
	}

	float* Engine::StagedCode(const Program& p)
	{
		return reinterpret_cast<float*>(static_cast<uint8_t*>(Staging) + LayoutOf(p).CodeOff);
	}

	cudaError_t Engine::RestageCode(const Program& p, cudaStream_t s)
	{
		const ProgramLayout l = LayoutOf(p);
		return cudaMemcpyAsync(static_cast<uint8_t*>(ProgramScratch.Ptr) + l.CodeOff, static_cast<uint8_t*>(Staging) + l.CodeOff,
			l.CodeBytes, cudaMemcpyHostToDevice, s);
	}

	// One allocation: nodes (64-byte records), code quads, colour bytes, material RGB.
	cudaError_t Engine::Upload(Program& p)
	{
		const ProgramLayout l = LayoutOf(p);
		cudaError_t e = cudaGetDevice(&p.DeviceId);
		if (e != cudaSuccess) return e;
		e = cudaMalloc(&p.Device, l.Total);
		if (e != cudaSuccess) { p.Device = nullptr; return e; }
		std::vector<uint8_t> staging(l.Total, 0);
		Pack(p, l, staging.data());
		e = cudaMemcpy(p.Device, staging.data(), l.Total, cudaMemcpyHostToDevice);
		if (e != cudaSuccess) return e;
		Bind(p, l, p.Device);
		return cudaSuccess;
	}

	void Engine::SetProfiling(bool on) { Profiling = on; }

	void Engine::ResetProfile()
	{
		Collect();
		Totals.clear();
	}

	void Engine::Begin(const char* name, cudaStream_t s)
	{
		if (!Profiling) return;
		Mark m{ name, nullptr, nullptr };
		cudaEventCreate(&m.Start);
		cudaEventCreate(&m.Stop);
		cudaEventRecord(m.Start, s);
		Pending.push_back(m);
	}

	void Engine::End(cudaStream_t s)
	{
		if (!Profiling || Pending.empty()) return;
		cudaEventRecord(Pending.back().Stop, s);
	}

	void Engine::Collect()
	{
		for (Mark& m : Pending)
		{
			float ms = 0.0f;
			if (cudaEventSynchronize(m.Stop) == cudaSuccess) cudaEventElapsedTime(&ms, m.Start, m.Stop);
			cudaEventDestroy(m.Start);
			cudaEventDestroy(m.Stop);
			bool found = false;
			for (Total& t : Totals)
			{
				if (t.Name == m.Name) { t.Ms += ms; t.Launches += 1; found = true; break; }
			}
			if (!found) Totals.push_back({ m.Name, (double)ms, 1 });
		}
		Pending.clear();
	}

	bool Engine::ReadProfile(const std::string& name, double& ms, int64_t& launches)
	{
		Collect();
		for (const Total& t : Totals)
		{
			if (t.Name == name) { ms = t.Ms; launches = t.Launches; return true; }
		}
		ms = 0.0;
		launches = 0;
		return false;
	}

#define TG_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return _e; } while (0)

	cudaError_t Engine::EvalGrid(const Program& p, const GridSpec& g, float* out, cudaStream_t s)
	{
		Begin("eval_grid", s);
		cudaError_t e = LaunchEvalGrid(p.View, g, out, s);
		End(s);
		return e;
	}

	cudaError_t Engine::EvalPoints(const Program& p, const float* host_points, int64_t n, float* host_out, cudaStream_t s)
	{
		if (n <= 0) return cudaSuccess;
		TG_TRY(Points.Reserve((size_t)n * 12));
		TG_TRY(PointOut.Reserve((size_t)n * 4));
		TG_TRY(cudaMemcpyAsync(Points.Ptr, host_points, (size_t)n * 12, cudaMemcpyHostToDevice, s));
		Begin("eval_points", s);
		TG_TRY(LaunchEvalPoints(p.View, Points.As<float>(), n, PointOut.As<float>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(host_out, PointOut.Ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		Collect();
		return cudaSuccess;
	}

	cudaError_t Engine::PreClassify(const RootProgram& root, const GridSpec& g, int B, cudaStream_t s)
	{
		PreValid = false;
		if (B < 1 || B > 32 || root.Code.empty()) return cudaErrorInvalidValue;
		const int64_t nb = BrickCount(g, B);
		if (nb <= 0) return cudaErrorInvalidValue;
		TG_TRY(BrickBits.Reserve((size_t)((nb + 31) / 32) * 4));
		// One node (64 bytes), then the records at a 256-byte boundary, as Pack lays out a
		// program.
		const size_t codeOff = 256, total = codeOff + root.Code.size() * sizeof(float);
		TG_TRY(RootScratch.Reserve(total));
		if (RootCopyPending)
		{
			TG_TRY(cudaEventSynchronize(RootCopied));
			RootCopyPending = false;
		}
		if (RootStagingBytes < total)
		{
			if (RootStaging) cudaFreeHost(RootStaging);
			RootStaging = nullptr;
			RootStagingBytes = 0;
			TG_TRY(cudaMallocHost(&RootStaging, total + total / 4));
			RootStagingBytes = total + total / 4;
		}
		uint8_t* st = static_cast<uint8_t*>(RootStaging);
		std::memcpy(st, &root.Node, sizeof(OctNode));
		std::memcpy(st + codeOff, root.Code.data(), root.Code.size() * sizeof(float));
		if (!RootCopied) TG_TRY(cudaEventCreateWithFlags(&RootCopied, cudaEventDisableTiming));
		TG_TRY(cudaMemcpyAsync(RootScratch.Ptr, RootStaging, total, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaEventRecord(RootCopied, s));
		RootCopyPending = true;
		DeviceProgram v{};
		v.Nodes = RootScratch.As<OctNode>();
		v.Code = reinterpret_cast<const float4*>(RootScratch.As<uint8_t>() + codeOff);
		v.MaxStack = root.Node.StackSize;
		v.Lipschitz = root.Node.ClipRadius >= 0.0f ? 1 : 0;
		Begin("classify_root", s);
		TG_TRY(LaunchClassifyBricks(v, g, B, BrickBits.As<uint32_t>(), s));
		End(s);
		PreValid = true;
		PreGrid = g;
		PreBrickSize = B;
		return cudaSuccess;
	}

	cudaError_t Engine::Export(const Program& p, const GridSpec& g, const ExportOptions& opt, DeviceMesh& out, cudaStream_t s)
	{
		// Bits PreClassify left for this export (any other export voids them).
		const bool pre = opt.PreClassified && PreValid && !opt.Dense && !opt.Field && PreBrickSize == opt.BrickSize &&
			std::memcmp(&PreGrid, &g, sizeof(GridSpec)) == 0;
		PreValid = false;
		// A code copy RestageCode started reads the staging buffer: whatever way this export
		// ends, it is over before the next upload rewrites that buffer.
		struct RestageWait
		{
			cudaEvent_t Event = nullptr;
			~RestageWait() { if (Event) cudaEventSynchronize(Event); }
		} restaged;
		out = DeviceMesh();
		// Asynchronous exports stop at a synchronisation point once cancelled.
		auto stopped = [&](float done) -> bool
		{
			if (opt.Progress) opt.Progress->store(done);
			if (opt.Active && !opt.Active->load())
			{
				if (opt.Cancelled) *opt.Cancelled = true;
				return true;
			}
			return false;
		};
		const int64_t lattice = (int64_t)g.NX * g.NY * g.NZ;
		const int64_t cells = (int64_t)(g.NX - 1) * (g.NY - 1) * (g.NZ - 1);
		const int64_t words = (cells + 31) / 32;
		if (!HostCounts) TG_TRY(cudaMallocHost(&HostCounts, 8 * sizeof(uint32_t)));

		TG_TRY(LatticeBuf.Reserve((size_t)lattice * sizeof(float)));
		TG_TRY(Words.Reserve((size_t)words * 4));
		TG_TRY(WordBase.Reserve((size_t)words * 4));
		TG_TRY(Counts.Reserve(8 * sizeof(uint32_t)));
		TG_TRY(Scratch.Reserve(ScanScratchWords(words) * 4));

		if (opt.Dense)
		{
			Bricks = ActiveBricks = 0;
			Begin("eval_grid", s);
			TG_TRY(LaunchEvalGrid(p.View, g, LatticeBuf.As<float>(), s, opt.Lanes));
			End(s);
			Begin("cell_flags", s);
			TG_TRY(LaunchCellFlags(LatticeBuf.As<float>(), g, Words.As<uint32_t>(), s));
			End(s);
		}
		else
		{
			const int B = opt.BrickSize;
			const int64_t nb = BrickCount(g, B);
			const int64_t brickWords = (nb + 31) / 32;
			TG_TRY(BrickBits.Reserve((size_t)brickWords * 4 * (opt.Field && opt.Refine ? 2 : 1)));
			TG_TRY(BrickList.Reserve((size_t)nb * 4));
			TG_TRY(BrickTops.Reserve((size_t)nb * 4));
			// The exact classifier stores each kept brick's descent for the evaluation; the
			// network alone leaves the evaluation to descend.
			uint32_t* tops = (!opt.Field || opt.Refine) ? BrickTops.As<uint32_t>() : nullptr;
			if (!SmCount)
			{
				int dev = 0;
				TG_TRY(cudaGetDevice(&dev));
				TG_TRY(cudaDeviceGetAttribute(&SmCount, cudaDevAttrMultiProcessorCount, dev));
			}
			uint32_t* brickCount = Counts.As<uint32_t>() + 2;
			uint32_t* bits = BrickBits.As<uint32_t>();
			if (opt.Field)
			{
				// Ball radius of a whole brick: half its diagonal.
				const float radius = 0.8660254f * (float)B * std::max(g.DX, std::max(g.DY, g.DZ));
				Begin("classify_field", s);
				TG_TRY(LaunchFieldClassifyBricks(p.View, g, B, opt.Field->Grid, opt.Field->TablePtr(), opt.Field->ImagePtr(),
					opt.Field->MarginFor(radius), bits, opt.Field->StatusPtr(), s));
				End(s);
				if (opt.Refine)
				{
					// The exact test on the bricks the network kept, in the classifier's
					// spatial tiles; survivors go to the second half of the bit buffer.
					uint32_t* kept = bits + brickWords;
					Begin("refine_bricks", s);
					TG_TRY(LaunchClassifyBricks(p.View, g, B, kept, s, bits, BrickTops.As<uint32_t>()));
					End(s);
					bits = kept;
				}
			}
			else if (!pre)
			{
				Begin("classify_bricks", s);
				TG_TRY(LaunchClassifyBricks(p.View, g, B, bits, s, nullptr, BrickTops.As<uint32_t>()));
				End(s);
			}
			Begin("list_bricks", s);
			TG_TRY(ClassCounts.Reserve(8 * sizeof(uint32_t)));
			TG_TRY(LaunchListBricks(bits, nb, WordBase.As<uint32_t>(), Scratch.As<uint32_t>(), BrickList.As<uint32_t>(), brickCount, s,
				&p.View, tops, ClassCounts.As<uint32_t>(), pre ? &g : nullptr, B));
			End(s);
			LastBrickSize = B;
			// Active cells lie in listed bricks: bound the list by the bricks' cells.
			TG_TRY(ActiveCells.Reserve((size_t)(nb * (int64_t)B * B * B < cells ? nb * (int64_t)B * B * B : cells) * 4));
			int* evalStatus = reinterpret_cast<int*>(Counts.As<uint32_t>() + 4);      // status and work counter
			TG_TRY(cudaMemsetAsync(evalStatus, 0, 2 * sizeof(int), s));
			if (B == 7 && !opt.Staged)
			{
				// The cell pass runs inside the brick evaluation, on each brick's values in
				// shared memory.
				Begin("eval_bricks", s);
				TG_TRY(LaunchEvalBricksCells(p.View, g, BrickList.As<uint32_t>(), brickCount, tops, LatticeBuf.As<float>(),
					Words.As<uint32_t>(), ActiveCells.As<uint32_t>(), Counts.As<uint32_t>() + 3, SmCount, s, opt.Lanes, evalStatus));
				End(s);
			}
			else
			{
				Begin("eval_bricks", s);
				TG_TRY(LaunchEvalBricks(p.View, g, B, BrickList.As<uint32_t>(), brickCount, tops, LatticeBuf.As<float>(), SmCount, s,
					opt.Lanes, opt.Staged, evalStatus));
				End(s);
				Begin("cell_flags", s);
				TG_TRY(LaunchCellFlagsListed(LatticeBuf.As<float>(), g, B, BrickList.As<uint32_t>(), brickCount, Words.As<uint32_t>(),
					ActiveCells.As<uint32_t>(), Counts.As<uint32_t>() + 3, SmCount, s));
				End(s);
			}
			TG_TRY(cudaMemcpyAsync(HostCounts + 2, brickCount, 12, cudaMemcpyDeviceToHost, s));
			Bricks = nb;
		}
		Begin("scan", s);
		TG_TRY(LaunchExclusiveScan(Words.As<uint32_t>(), words, true, WordBase.As<uint32_t>(), Counts.As<uint32_t>(), Scratch.As<uint32_t>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(HostCounts, Counts.Ptr, 4, cudaMemcpyDeviceToHost, s));
		if (opt.WhileWaiting) TG_TRY(opt.WhileWaiting());
		TG_TRY(cudaStreamSynchronize(s));
		if (opt.RestageCode)
		{
			// The kernels that read distance programs are done; the ones up to the attribute
			// pass read no program, so the copy runs beside them.
			if (!CopyStream) TG_TRY(cudaStreamCreateWithFlags(&CopyStream, cudaStreamNonBlocking));
			if (!CodeReady) TG_TRY(cudaEventCreateWithFlags(&CodeReady, cudaEventDisableTiming));
			TG_TRY(RestageCode(p, CopyStream));
			TG_TRY(cudaEventRecord(CodeReady, CopyStream));
			restaged.Event = CodeReady;
		}
		const uint32_t vcount = HostCounts[0];
		if (!opt.Dense) ActiveBricks = HostCounts[2];
		if (!opt.Dense && HostCounts[4] != 0)
		{
			SetError("brick evaluation: a program copy to shared memory did not complete in time");
			return cudaErrorLaunchTimeout;
		}
		if (stopped(0.6f)) return cudaSuccess;

		TG_TRY(Vertices.Reserve((size_t)vcount * 12));
		TG_TRY(Cubes.Reserve((size_t)vcount * 4));
		TG_TRY(FaceCounts.Reserve((size_t)vcount * 4));
		TG_TRY(FaceBase.Reserve((size_t)vcount * 4));
		TG_TRY(Scratch.Reserve(ScanScratchWords(vcount) * 4));
		Begin("cell_vertices", s);
		if (opt.Dense)
		{
			TG_TRY(LaunchCellVertices(LatticeBuf.As<float>(), g, Words.As<uint32_t>(), WordBase.As<uint32_t>(), Vertices.As<float>(),
				Cubes.As<uint32_t>(), FaceCounts.As<uint32_t>(), cells, s));
		}
		else
		{
			TG_TRY(LaunchCellVerticesListed(LatticeBuf.As<float>(), g, ActiveCells.As<uint32_t>(), HostCounts[3], Words.As<uint32_t>(),
				WordBase.As<uint32_t>(), Vertices.As<float>(), Cubes.As<uint32_t>(), FaceCounts.As<uint32_t>(), s));
		}
		End(s);
		Begin("scan", s);
		TG_TRY(LaunchExclusiveScan(FaceCounts.As<uint32_t>(), vcount, false, FaceBase.As<uint32_t>(), Counts.As<uint32_t>() + 1,
			Scratch.As<uint32_t>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(HostCounts + 1, Counts.As<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		const uint32_t fcount = HostCounts[1];
		if (stopped(0.8f)) return cudaSuccess;

		TG_TRY(Faces.Reserve((size_t)fcount * 12));
		Begin("faces", s);
		TG_TRY(LaunchFaces(LatticeBuf.As<float>(), g, Words.As<uint32_t>(), WordBase.As<uint32_t>(), Cubes.As<uint32_t>(),
			FaceBase.As<uint32_t>(), vcount, Faces.As<uint32_t>(), s));
		End(s);

		out.VertexCount = vcount;
		out.FaceCount = fcount;
		out.Vertices = Vertices.As<float>();
		out.Cubes = Cubes.As<uint32_t>();
		out.Faces = Faces.As<uint32_t>();
		HostMeshOut* host = opt.Host;
		bool early = false;
		if (host)
		{
			// Host blocks now that the counts are known; vertices, cubes and faces travel on
			// the copy stream while the attribute pass runs.
			*host = HostMeshOut();
			host->VertexCount = vcount;
			host->FaceCount = fcount;
			const size_t v = vcount ? vcount : 1, f = fcount ? fcount : 1;
			auto take = [](size_t bytes) -> void*
			{
				void* b = HostPool::Get().Take(bytes);
				return b ? b : std::malloc(bytes);
			};
			host->Vertices = (float*)take(v * 12);
			host->Normals = (float*)take(v * 12);
			host->Faces = (uint32_t*)take(f * 12);
			host->Cubes = (uint32_t*)take(v * 4);
			if (opt.Attributes && p.Host.Header.HasPaint) host->Colors = (uint8_t*)take(v * 3);
			if (!host->Vertices || !host->Normals || !host->Faces || !host->Cubes ||
				(opt.Attributes && p.Host.Header.HasPaint && !host->Colors))
			{
				FreeHostMesh(*host);
				host->OutOfMemory = true;
				host = nullptr;
			}
			else
			{
				if (!CopyStream) TG_TRY(cudaStreamCreateWithFlags(&CopyStream, cudaStreamNonBlocking));
				if (!MeshReady) TG_TRY(cudaEventCreateWithFlags(&MeshReady, cudaEventDisableTiming));
				TG_TRY(cudaEventRecord(MeshReady, s));
				TG_TRY(cudaStreamWaitEvent(CopyStream, MeshReady, 0));
				if (vcount)
				{
					TG_TRY(cudaMemcpyAsync(host->Vertices, Vertices.Ptr, (size_t)vcount * 12, cudaMemcpyDeviceToHost, CopyStream));
					TG_TRY(cudaMemcpyAsync(host->Cubes, Cubes.Ptr, (size_t)vcount * 4, cudaMemcpyDeviceToHost, CopyStream));
				}
				if (fcount) TG_TRY(cudaMemcpyAsync(host->Faces, Faces.Ptr, (size_t)fcount * 12, cudaMemcpyDeviceToHost, CopyStream));
				early = true;
			}
		}
		if (opt.Attributes)
		{
			TG_TRY(Normals.Reserve((size_t)vcount * 12));
			uint8_t* colors = nullptr;
			if (p.Host.Header.HasPaint)
			{
				TG_TRY(Colors.Reserve((size_t)vcount * 3));
				colors = Colors.As<uint8_t>();
			}
			// The culled export visits the vertices in its active-cell list's order (cells
			// grouped by brick, so a warp's vertices mostly share one surface program).
			VertexOrder order;
			if (!opt.Dense) order = { ActiveCells.As<uint32_t>(), Words.As<uint32_t>(), WordBase.As<uint32_t>() };
			if (restaged.Event) TG_TRY(cudaStreamWaitEvent(s, restaged.Event, 0));
			Begin("attributes", s);
			TG_TRY(LaunchVertexAttributes(p.View, Vertices.As<float>(), vcount, Normals.As<float>(), colors, s, order));
			End(s);
			out.Normals = Normals.As<float>();
			out.Colors = colors;
			if (early && vcount)
			{
				TG_TRY(cudaMemcpyAsync(host->Normals, Normals.Ptr, (size_t)vcount * 12, cudaMemcpyDeviceToHost, s));
				if (colors) TG_TRY(cudaMemcpyAsync(host->Colors, colors, (size_t)vcount * 3, cudaMemcpyDeviceToHost, s));
			}
		}
		else if (early)
		{
			std::memset(host->Normals, 0, (size_t)(vcount ? vcount : 1) * 12);
		}
		TG_TRY(cudaStreamSynchronize(s));
		if (early) TG_TRY(cudaStreamSynchronize(CopyStream));
		Collect();
		if (opt.Field) TG_TRY(const_cast<FieldNet*>(opt.Field)->CheckStatus(s));
		if (opt.Progress) opt.Progress->store(1.0f);
		return cudaSuccess;
	}

	void FreeHostMesh(HostMeshOut& m)
	{
		void* blocks[5] = { m.Vertices, m.Normals, m.Colors, m.Faces, m.Cubes };
		for (void* b : blocks)
		{
			if (b && !HostPool::Get().Give(b)) std::free(b);
		}
		m = HostMeshOut();
	}

	cudaError_t Engine::LastBrickList(std::vector<uint32_t>& out, int& brick_size)
	{
		out.resize((size_t)ActiveBricks);
		brick_size = LastBrickSize;
		if (ActiveBricks <= 0) return cudaSuccess;
		TG_TRY(cudaMemcpy(out.data(), BrickList.Ptr, (size_t)ActiveBricks * 4, cudaMemcpyDeviceToHost));
		std::sort(out.begin(), out.end());      // the evaluation's list is in cost order
		return cudaSuccess;
	}

	cudaError_t Engine::FaceNormals(const Program& p, const float* host_vertices, uint64_t vertex_count, const uint32_t* host_faces,
		uint64_t face_count, float* host_normals, cudaStream_t s)
	{
		if (face_count == 0) return cudaSuccess;
		DeviceBuffer v, f, n;
		TG_TRY(v.Reserve(vertex_count * 12));
		TG_TRY(f.Reserve(face_count * 12));
		TG_TRY(n.Reserve(face_count * 12));
		cudaError_t e = cudaMemcpyAsync(v.Ptr, host_vertices, vertex_count * 12, cudaMemcpyHostToDevice, s);
		if (e == cudaSuccess) e = cudaMemcpyAsync(f.Ptr, host_faces, face_count * 12, cudaMemcpyHostToDevice, s);
		Begin("face_normals", s);
		if (e == cudaSuccess) e = LaunchFaceNormals(p.View, v.As<float>(), f.As<uint32_t>(), face_count, n.As<float>(), s);
		End(s);
		if (e == cudaSuccess) e = cudaMemcpyAsync(host_normals, n.Ptr, face_count * 12, cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		Collect();
		v.Release(); f.Release(); n.Release();
		return e;
	}

	cudaError_t Engine::RayMarch(const Program& p, const float* origins, const float* dirs, int64_t n, int iterations, float epsilon,
		uint8_t* hit, float* travel, float* position, cudaStream_t s, const RayFrame* frame)
	{
		if (n <= 0) return cudaSuccess;
		const size_t in = (size_t)n * 12;
		TG_TRY(RayIn.Reserve(2 * in));
		TG_TRY(RayOut.Reserve((size_t)n * 17));
		float* dOrig = RayIn.As<float>();
		float* dDir = dOrig + n * 3;
		float* dTravel = RayOut.As<float>();
		float* dPos = dTravel + n;
		uint8_t* dHit = reinterpret_cast<uint8_t*>(dPos + n * 3);
		TG_TRY(cudaMemcpyAsync(dOrig, origins, in, cudaMemcpyHostToDevice, s));
		TG_TRY(cudaMemcpyAsync(dDir, dirs, in, cudaMemcpyHostToDevice, s));
		Begin("ray_march", s);
		if (frame && frame->Mode != 0) TG_TRY(LaunchRayQuery(p.View, *frame, dOrig, dDir, n, iterations, epsilon, dHit, dTravel, dPos, s));
		else TG_TRY(LaunchRayMarch(p.View, dOrig, dDir, n, iterations, epsilon, dHit, dTravel, dPos, s));
		End(s);
		TG_TRY(cudaMemcpyAsync(hit, dHit, (size_t)n, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaMemcpyAsync(travel, dTravel, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaMemcpyAsync(position, dPos, in, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		Collect();
		return cudaSuccess;
	}

	cudaError_t Engine::PointQuery(const Program& p, const float* points, int64_t n, bool gradient, float* out, cudaStream_t s)
	{
		if (n <= 0) return cudaSuccess;
		const size_t in = (size_t)n * 12, outBytes = (size_t)n * (gradient ? 12 : 4);
		TG_TRY(RayIn.Reserve(in));
		TG_TRY(RayOut.Reserve(outBytes));
		TG_TRY(cudaMemcpyAsync(RayIn.Ptr, points, in, cudaMemcpyHostToDevice, s));
		Begin(gradient ? "tree_gradient" : "tree_eval", s);
		TG_TRY(LaunchPointQuery(p.View, RayIn.As<float>(), n, gradient, RayOut.As<float>(), s));
		End(s);
		TG_TRY(cudaMemcpyAsync(out, RayOut.Ptr, outBytes, cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		Collect();
		return cudaSuccess;
	}

	cudaError_t Engine::Render(const Program& p, const CameraBasis* cams, int count, int width, int height, int steps, float epsilon,
		bool exact, float* depth, float* normals, uint8_t* colors, bool out_is_device, cudaStream_t s, const FieldNet* field)
	{
		const int64_t px = (int64_t)width * height * count;
		if (px <= 0) return cudaSuccess;
		TG_TRY(Cameras.Reserve(sizeof(CameraBasis) * (size_t)count));
		TG_TRY(cudaMemcpyAsync(Cameras.Ptr, cams, sizeof(CameraBasis) * (size_t)count, cudaMemcpyHostToDevice, s));
		float* dDepth = depth;
		float* dNormals = normals;
		uint8_t* dColors = colors;
		if (!out_is_device)
		{
			TG_TRY(Image.Reserve((size_t)px * (4 + 12 + 3)));
			dDepth = Image.As<float>();
			dNormals = dDepth + px;
			dColors = colors ? reinterpret_cast<uint8_t*>(dNormals + px * 3) : nullptr;
		}
		if (field)
		{
			TG_TRY(RenderCounters.Reserve(2 * sizeof(unsigned long long)));
			TG_TRY(cudaMemsetAsync(RenderCounters.Ptr, 0, 2 * sizeof(unsigned long long), s));
			// Network steps stop within a few network margins of the surface; exact steps finish.
			const float margin = field->Info.MarginOverride >= 0.0f ? field->Info.MarginOverride : field->Info.Margin;
			const float switchAt = margin > epsilon ? margin : epsilon;
			TG_TRY(RayIn.Reserve((size_t)px * 8));
			Begin("render_field", s);
			TG_TRY(LaunchRenderField(p.View, Cameras.As<CameraBasis>(), count, width, height, steps, epsilon, field->Grid,
				field->TablePtr(), field->ImagePtr(), margin, switchAt, RayIn.As<float>(), RayIn.As<uint32_t>() + px, dDepth, dNormals,
				dColors, RenderCounters.As<unsigned long long>(), field->StatusPtr(), s));
			End(s);
		}
		else
		{
			Begin("render", s);
			TG_TRY(LaunchRender(p.View, Cameras.As<CameraBasis>(), count, width, height, steps, epsilon, exact, dDepth, dNormals, dColors, s));
			End(s);
		}
		if (!out_is_device)
		{
			TG_TRY(cudaMemcpyAsync(depth, dDepth, (size_t)px * 4, cudaMemcpyDeviceToHost, s));
			TG_TRY(cudaMemcpyAsync(normals, dNormals, (size_t)px * 12, cudaMemcpyDeviceToHost, s));
			if (colors) TG_TRY(cudaMemcpyAsync(colors, dColors, (size_t)px * 3, cudaMemcpyDeviceToHost, s));
		}
		TG_TRY(cudaStreamSynchronize(s));
		Collect();
		if (field)
		{
			unsigned long long c[2] = { 0, 0 };
			TG_TRY(cudaMemcpy(c, RenderCounters.Ptr, sizeof c, cudaMemcpyDeviceToHost));
			LastNetworkSteps = c[0];
			LastExactSteps = c[1];
			TG_TRY(const_cast<FieldNet*>(field)->CheckStatus(s));
		}
		return cudaSuccess;
	}
}
