// Host-callable launchers for the export kernels.  All take device pointers and a
// stream and return a cudaError_t; none allocates.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../host/tg_layout.hpp"

namespace tg
{
	struct DeviceProgram
	{
		const OctNode* Nodes;
		const float4* Code;
		const uchar4* Colors;
		int MaxStack;
		int FullSurfaceCode;    // the whole tree's surface program
		int Lipschitz;          // every brush 1-Lipschitz
	};

	// Pinhole camera: pixel (x, y) looks along forward + right*u + up*v with
	// u = (2(x + 0.5)/W - 1) * tan_half_fov * W/H and v = (1 - 2(y + 0.5)/H) * tan_half_fov.
	struct CameraBasis
	{
		float Position[3];
		float Forward[3];
		float Right[3];
		float Up[3];
		float TanHalfFov;
		float Aspect;
	};

	// SDFNode::RayMarch on the whole tree for n rays (reference step sequence).
	cudaError_t LaunchRayMarch(const DeviceProgram& prog, const float* origins, const float* dirs, int64_t n, int max_iterations,
		float epsilon, uint8_t* hit, float* travel, float* position, cudaStream_t stream);

	// Depth (travel, +inf on a miss), gradient normal and colour per pixel for `count`
	// cameras.  exact: the reference's full-tree steps; otherwise octree-bounded steps.
	cudaError_t LaunchRender(const DeviceProgram& prog, const CameraBasis* cameras, int count, int width, int height,
		int max_steps, float epsilon, bool exact, float* depth, float* normals, uint8_t* colors, cudaStream_t stream);

	// Distances at every lattice point (x fastest), SDFOctree::Eval(p, Exact = true).
	// `lanes` points per thread (1, 2 or 4) share one pass over the records.
	cudaError_t LaunchEvalGrid(const DeviceProgram& prog, const GridSpec& grid, float* out, cudaStream_t stream, int lanes = 4);

	// Surface nets, cell pass part 1: one bit per cell (x fastest) set when the cell's
	// eight corners do not all share a sign.  `words` holds ceil(cells / 32) words.
	cudaError_t LaunchCellFlags(const float* lattice, const GridSpec& grid, uint32_t* words, cudaStream_t stream);

	// Exact brick culling (tg_cull.cu): bricks of B^3 cells that provably hold no sign
	// change are skipped.  brick_bits: one bit per brick; list/count: surviving bricks.
	int64_t BrickCount(const GridSpec& g, int B);
	cudaError_t LaunchClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, uint32_t* brick_bits, uint32_t* list,
		uint32_t* count, cudaStream_t stream);
	cudaError_t LaunchEvalBricks(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		float* lattice, int grid_blocks, cudaStream_t stream, int lanes = 4);
	cudaError_t LaunchCellFlagsBricks(const float* lattice, const GridSpec& g, int B, const uint32_t* brick_bits, uint32_t* words,
		cudaStream_t stream);
	// Cell pass over the cells of listed bricks only: clears and fills the bitmask and
	// lists the active cells (`cells` holds up to the lattice's cell count).
	cudaError_t LaunchCellFlagsListed(const float* lattice, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		uint32_t* words, uint32_t* cells, uint32_t* cell_count, int grid_blocks, cudaStream_t stream);
	// Vertex pass over the listed active cells (one thread each).
	cudaError_t LaunchCellVerticesListed(const float* lattice, const GridSpec& g, const uint32_t* cells, uint32_t cell_count,
		const uint32_t* words, const uint32_t* word_base, float* vertices, uint32_t* cubes, uint32_t* face_counts, cudaStream_t stream);

	// Exclusive prefix sum of popcount(words[i]) (popcount = true) or of counts[i].
	// `scratch` needs ScanScratchWords(n) words.  `total` (device) receives the sum.
	size_t ScanScratchWords(int64_t n);
	cudaError_t LaunchExclusiveScan(const uint32_t* in, int64_t n, bool popcount, uint32_t* out, uint32_t* total,
		uint32_t* scratch, cudaStream_t stream);

	// Cell pass part 2: vertex of every active cell at its rank (cell order), its cube
	// index, and how many triangles the face pass will emit for it.
	cudaError_t LaunchCellVertices(const float* lattice, const GridSpec& grid, const uint32_t* words, const uint32_t* word_base,
		float* vertices, uint32_t* cubes, uint32_t* face_counts, int64_t cells, cudaStream_t stream);

	// Face pass: triangles (v0, v1, v2) per active cell, at face_base[vertex].
	cudaError_t LaunchFaces(const float* lattice, const GridSpec& grid, const uint32_t* words, const uint32_t* word_base,
		const uint32_t* cubes, const uint32_t* face_base, uint32_t vertex_count, uint32_t* faces, cudaStream_t stream);

	// Octree distances at arbitrary points (3 floats per point).
	cudaError_t LaunchEvalPoints(const DeviceProgram& prog, const float* points, int64_t n, float* out, cudaStream_t stream);

	// Gradient normal at each triangle's centroid, as WriteSTL(Octree, ...) writes it.
	cudaError_t LaunchFaceNormals(const DeviceProgram& prog, const float* vertices, const uint32_t* faces, uint64_t face_count,
		float* normals, cudaStream_t stream);

	// Achieved FP32 fused-multiply-add throughput of this GPU (TFLOP/s, 2 flops per FMA).
	cudaError_t MeasureFp32Peak(double* tflops, cudaStream_t stream);

	// Gradient normal and colour bytes per vertex (SDFOctree::Gradient / GetMaterial).
	cudaError_t LaunchVertexAttributes(const DeviceProgram& prog, const float* vertices, uint32_t vertex_count,
		float* normals, uint8_t* colors, cudaStream_t stream);
}
