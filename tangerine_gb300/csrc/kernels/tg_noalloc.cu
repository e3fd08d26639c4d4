// tg_export_mesh_noalloc: the mesh export for callers that must not allocate GPU memory.
//
// Some callers cannot call cudaMalloc once they are running: a host application that
// hands all device memory to its own pool at start-up, or meshing code on a latency-bound
// thread where cudaMalloc/cudaFree's implicit device-wide synchronisation is not
// acceptable.  This entry point runs the dense export kernels (every lattice point
// evaluated, as the reference does -- not tg_export_mesh's default brick-culled path; the
// mesh is the same bit for bit), with the export's scratch memory -- the lattice of
// distances, the active-cell bitmask, its prefix sums, the per-vertex triangle counts and
// the scan block sums -- in one file-scope device array of fixed size
// (kNoAllocScratchBytes, 64 MiB), and output buffers the caller passes.  The library never
// allocates on this path.
//
// * The array belongs to this file's CUDA module.  CUDA loads modules lazily (the default
//   since CUDA 12.2), so a device reserves the 64 MiB the first time this entry point
//   runs on it -- at the set-up call (program and grid NULL) or the first export -- and
//   holds them until the process exits.  A caller that later gives the rest of device
//   memory to its own pool makes that first call before it does.
// * The array's device address is looked up with cudaGetSymbolAddress by that first call
//   on a device (with that device current) and cached; make that first call before any
//   stream capture.  cudaDeviceReset invalidates the cached address: it is not supported
//   while the library is in use.
// * All calls share the array and it keeps the last call's contents.  The pipeline writes
//   every scratch word before reading it; the vertex/face totals are cleared each call.
//   Calls that overlap on the GPU (from several host threads or streams) race on the
//   array: serialise them.
#include <mutex>

#include "tg_kernels.hpp"
#include "../host/tg_engine.hpp"
#include "../../../include/tangerine_gb300.h"

namespace tg
{
	namespace
	{
		constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
		constexpr int kMaxDevices = 64;

		__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

		std::mutex g_setup_mutex;
		void* g_scratch_address[kMaxDevices] = {};

		// Device address of the scratch array on `device` (must be current).
		cudaError_t ScratchAddress(int device, void** out)
		{
			if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
			std::lock_guard<std::mutex> lock(g_setup_mutex);
			if (!g_scratch_address[device])
			{
				void* p = nullptr;
				const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
				if (e != cudaSuccess) return e;
				g_scratch_address[device] = p;
			}
			*out = g_scratch_address[device];
			return cudaSuccess;
		}

		inline size_t Align256(size_t v) { return (v + 255) / 256 * 256; }

		tg_status Fail(tg_status st, const std::string& msg)
		{
			SetError(msg);
			return st;
		}

		tg_status CudaFail(cudaError_t e, const char* what)
		{
			SetError(std::string(what) + ": " + cudaGetErrorString(e));
			return TG_ERR_CUDA;
		}
	}
}

using namespace tg;

extern "C" TANGERINE_API tg_status tg_export_mesh_noalloc(tg_program* program, const tg_grid* grid, uint32_t flags,
	float* vertices, float* normals, uint8_t* colors, uint32_t* faces, uint32_t* cubes,
	uint64_t vertex_capacity, uint64_t face_capacity, uint64_t* counts, void* stream)
{
	if (!program && !grid && !vertices && !normals && !colors && !faces && !cubes && !counts)
	{
		// Set-up only: reserve the scratch array on the current device and cache its address.
		int device = 0;
		cudaError_t e = cudaGetDevice(&device);
		if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: cudaGetDevice");
		void* base = nullptr;
		e = ScratchAddress(device, &base);
		if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: cudaGetSymbolAddress");
		return TG_OK;
	}
	if (!program || !grid || !vertices || !faces || !cubes || !counts)
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: null argument");
	counts[0] = counts[1] = 0;
	if (flags & ~(uint32_t)(TG_MESH_ATTRIBUTES | TG_MESH_DENSE))
		return Fail(TG_ERR_UNSUPPORTED, "tg_export_mesh_noalloc: only TG_MESH_ATTRIBUTES and TG_MESH_DENSE apply "
			"(this path always evaluates every lattice point; brick and lane settings do not exist here)");
	const bool attributes = (flags & TG_MESH_ATTRIBUTES) != 0;
	if (attributes && !normals)
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: normals buffer required with TG_MESH_ATTRIBUTES");
	if (attributes && program->Host.Header.HasPaint && !colors)
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: colors buffer required: the tree has paint");
	const float dy = grid->step_y != 0.0f ? grid->step_y : grid->step;
	const float dz = grid->step_z != 0.0f ? grid->step_z : grid->step;
	if (grid->nx < 2 || grid->ny < 2 || grid->nz < 2 || !(grid->step > 0.0f) || !(dy > 0.0f) || !(dz > 0.0f) ||
		grid->nx > (1 << 20) || grid->ny > (1 << 20) || grid->nz > (1 << 20))
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: a lattice needs 2..2^20 points per axis and positive steps");

	const GridSpec g{ grid->x0, grid->y0, grid->z0, grid->step, dy, dz, (int)grid->nx, (int)grid->ny, (int)grid->nz };
	const int64_t lattice = grid->nx * grid->ny * grid->nz;
	const int64_t cells = (grid->nx - 1) * (grid->ny - 1) * (grid->nz - 1);
	const int64_t words = (cells + 31) / 32;
	const uint64_t vmax = vertex_capacity < (uint64_t)cells ? vertex_capacity : (uint64_t)cells;
	const int64_t scanItems = words > (int64_t)vmax ? words : (int64_t)vmax;

	// Scratch layout inside the static array.
	const size_t offLattice = 0;
	const size_t offWords = Align256(offLattice + (size_t)lattice * 4);
	const size_t offWordBase = Align256(offWords + (size_t)words * 4);
	const size_t offCounts = Align256(offWordBase + (size_t)words * 4);
	const size_t offScan = Align256(offCounts + 16);
	const size_t offFaceCounts = Align256(offScan + ScanScratchWords(scanItems) * 4);
	const size_t offFaceBase = Align256(offFaceCounts + (size_t)vmax * 4);
	const size_t need = Align256(offFaceBase + (size_t)vmax * 4);
	if (need > kNoAllocScratchBytes)
	{
		return Fail(TG_ERR_UNSUPPORTED, "tg_export_mesh_noalloc: this lattice needs " + std::to_string(need) +
			" bytes of scratch; the fixed scratch array holds " + std::to_string(kNoAllocScratchBytes) +
			" (use tg_export_mesh, or a smaller lattice or vertex capacity)");
	}

	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: cudaGetDevice");
	if (device != program->DeviceId)
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: the program was compiled for another device");
	void* base = nullptr;
	e = ScratchAddress(device, &base);
	if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: cudaGetSymbolAddress");

	unsigned char* s0 = static_cast<unsigned char*>(base);
	float* lat = reinterpret_cast<float*>(s0 + offLattice);
	uint32_t* wordBits = reinterpret_cast<uint32_t*>(s0 + offWords);
	uint32_t* wordBase = reinterpret_cast<uint32_t*>(s0 + offWordBase);
	uint32_t* totals = reinterpret_cast<uint32_t*>(s0 + offCounts);
	uint32_t* scan = reinterpret_cast<uint32_t*>(s0 + offScan);
	uint32_t* faceCounts = reinterpret_cast<uint32_t*>(s0 + offFaceCounts);
	uint32_t* faceBase = reinterpret_cast<uint32_t*>(s0 + offFaceBase);
	const cudaStream_t s = static_cast<cudaStream_t>(stream);

	uint32_t host[2] = { 0, 0 };
	e = cudaMemsetAsync(totals, 0, 16, s);
	if (e == cudaSuccess) e = LaunchEvalGrid(program->View, g, lat, s);
	if (e == cudaSuccess) e = LaunchCellFlags(lat, g, wordBits, s);
	if (e == cudaSuccess) e = LaunchExclusiveScan(wordBits, words, true, wordBase, totals, scan, s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&host[0], totals, 4, cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: cell pass");
	counts[0] = host[0];
	counts[1] = 0;
	if (host[0] > vertex_capacity)
	{
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: " + std::to_string(host[0]) +
			" vertices exceed the vertex capacity (counts[0] holds the size needed; counts[1] is known only "
			"once the vertices fit)");
	}

	e = LaunchCellVertices(lat, g, wordBits, wordBase, vertices, cubes, faceCounts, cells, s);
	if (e == cudaSuccess) e = LaunchExclusiveScan(faceCounts, host[0], false, faceBase, totals + 1, scan, s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&host[1], totals + 1, 4, cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: vertex pass");
	counts[1] = host[1];
	if (host[1] > face_capacity)
	{
		return Fail(TG_ERR_INVALID, "tg_export_mesh_noalloc: " + std::to_string(host[1]) +
			" faces exceed the face capacity (counts[1] holds the size needed)");
	}

	e = LaunchFaces(lat, g, wordBits, wordBase, cubes, faceBase, host[0], faces, s);
	if (e == cudaSuccess && attributes)
	{
		e = LaunchVertexAttributes(program->View, vertices, host[0], normals,
			program->Host.Header.HasPaint ? colors : nullptr, s);
	}
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return CudaFail(e, "tg_export_mesh_noalloc: face pass");
	return TG_OK;
}
