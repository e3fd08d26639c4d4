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
		const float4* MaterialRgb;  // stored RGB of each material, alpha 1
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
	// Ray frames of the app's casts: 0 plain SDFNode::RayMarch, 1 Lua's magnet cast (the
	// direction operand is a target), 2 SDFModel::RayMarch in a model frame.
	struct RayFrame
	{
		int Mode;
		float Rotation[4];      // w x y z
		float Translation[3];
		float Scale;
	};
	cudaError_t LaunchRayQuery(const DeviceProgram& prog, const RayFrame& frame, const float* origins, const float* dirs, int64_t n,
		int max_iterations, float epsilon, uint8_t* hit, float* travel, float* position, cudaStream_t stream);
	// SDFNode::Eval (1 float per point) or SDFNode::Gradient (3) on the whole tree.
	cudaError_t LaunchPointQuery(const DeviceProgram& prog, const float* points, int64_t n, bool gradient, float* out,
		cudaStream_t stream);

	cudaError_t LaunchRender(const DeviceProgram& prog, const CameraBasis* cameras, int count, int width, int height,
		int max_steps, float epsilon, bool exact, float* depth, float* normals, uint8_t* colors, cudaStream_t stream);

	// Distances at every lattice point (x fastest), SDFOctree::Eval(p, Exact = true).
	// `lanes` points per thread (1, 2 or 4) share one pass over the records.
	cudaError_t LaunchEvalGrid(const DeviceProgram& prog, const GridSpec& grid, float* out, cudaStream_t stream, int lanes = 4);

	// Surface nets, cell pass part 1: one bit per cell (x fastest) set when the cell's
	// eight corners do not all share a sign.  `words` holds ceil(cells / 32) words.
	cudaError_t LaunchCellFlags(const float* lattice, const GridSpec& grid, uint32_t* words, cudaStream_t stream);

	// Exact brick culling (tg_cull.cu): bricks of B^3 cells that provably hold no sign
	// change are skipped.  brick_bits: one bit per brick (set: may hold surface).
	int64_t BrickCount(const GridSpec& g, int B);
	// With `candidates` (bits of another classification, e.g. the learned bound's), only
	// bricks set there are tested; the rest stay clear.
	// brick_tops (optional, one word per brick): each kept brick's octree descent for the
	// evaluation (cell | shared << 31), which LaunchEvalBricks then reads instead of descending.
	cudaError_t LaunchClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, uint32_t* brick_bits, cudaStream_t stream,
		const uint32_t* candidates = nullptr, uint32_t* brick_tops = nullptr);
	// Set bits as a list in brick-index order (scan + compaction); *count (device) gets the
	// length.  base: (bricks + 31) / 32 words; scratch: ScanScratchWords of that.
	// With the classifier's brick_tops (and `prog`, and eight scratch words in class_counts),
	// the list is ordered instead by the cost of the bricks' programs, the costliest first,
	// so that a persistent evaluation does not end on them; base and scratch are then unused.
	// With `descend` (the export grid, and brick size B), the listing first writes each kept
	// brick's descent into `tops` itself (bits from a classification that stored none).
	cudaError_t LaunchListBricks(const uint32_t* brick_bits, int64_t bricks, uint32_t* base, uint32_t* scratch, uint32_t* list,
		uint32_t* count, cudaStream_t stream, const DeviceProgram* prog = nullptr, uint32_t* tops = nullptr,
		uint32_t* class_counts = nullptr, const GridSpec* descend = nullptr, int B = 0);
	// The brick kernels below run persistent grids sized from the SM count (`sms`).
	// Brick evaluation.  status[0..1], zeroed by the caller: status[0] becomes nonzero if a
	// staged program copy does not complete in time; status[1] is the warps' work counter.
	// staged: bricks inside one octree cell read their program from a shared-memory copy made
	// by one bulk copy.
	// tops: the classifier's brick_tops for every listed brick, or nullptr (the kernel descends).
	cudaError_t LaunchEvalBricks(const DeviceProgram& prog, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		const uint32_t* tops, float* lattice, int sms, cudaStream_t stream, int lanes, bool staged, int* status);
	// LaunchEvalBricks and LaunchCellFlagsListed in one launch, for 7^3-cell bricks with the
	// programs read from global memory: the same lattice, cell bits and active-cell list
	// (list order differs).  status as LaunchEvalBricks's.
	cudaError_t LaunchEvalBricksCells(const DeviceProgram& prog, const GridSpec& g, const uint32_t* list, const uint32_t* count,
		const uint32_t* tops, float* lattice, uint32_t* words, uint32_t* cells, uint32_t* cell_count, int sms, cudaStream_t stream,
		int lanes, int* status);
	cudaError_t LaunchCellFlagsBricks(const float* lattice, const GridSpec& g, int B, const uint32_t* brick_bits, uint32_t* words,
		cudaStream_t stream);
	// Cell pass over the cells of listed bricks only: clears and fills the bitmask and
	// lists the active cells (`cells` holds up to the lattice's cell count).
	cudaError_t LaunchCellFlagsListed(const float* lattice, const GridSpec& g, int B, const uint32_t* list, const uint32_t* count,
		uint32_t* words, uint32_t* cells, uint32_t* cell_count, int sms, cudaStream_t stream);
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

	// Self-check of the float blend-term evaluation against the double expression over n
	// seeded inputs (each both signs of the term): counts = checked, mismatches, fallbacks.
	cudaError_t LaunchBlendCheck(uint64_t n, uint64_t seed, unsigned long long* counts, cudaStream_t stream);
	// counts[0] = points checked, counts[1..9] = mismatches per check (tg_checks.cu).
	cudaError_t LaunchPairCheck(uint64_t n, uint64_t seed, unsigned long long* counts, cudaStream_t stream);

	// Test hooks of two bounded mbarrier waits (0 restores them): the staged-program copy of
	// the brick evaluation (tg_cull.cu) and the network-image copy of the field kernels
	// (tg_field.cu).  Nonzero, the wait is made on an mbarrier that nothing arrives at, with
	// this limit, so it runs out and the kernel takes its failure path.
	cudaError_t SetStageWaitTest(uint64_t limit_ns);
	cudaError_t SetSetupWaitTest(uint64_t limit_ns);

	// Achieved FP32 fused-multiply-add throughput of this GPU (TFLOP/s, 2 flops per FMA).
	cudaError_t MeasureFp32Peak(double* tflops, cudaStream_t stream);

	// The order the attribute passes visit the vertices in.  Cells == nullptr: vertex order.
	// Otherwise the active-cell list of the culled export (its cells grouped by brick): entry t
	// is the vertex of cell Cells[t], numbered as the cell passes number it (rank of the
	// cell's bit in Words, plus Base of its word).  Neighbouring cells mostly run one surface
	// program, so a warp visiting them in list order runs one program.
	struct VertexOrder
	{
		const uint32_t* Cells = nullptr;
		const uint32_t* Words = nullptr;
		const uint32_t* Base = nullptr;
	};

	// Gradient normal and colour bytes per vertex (SDFOctree::Gradient / GetMaterial).
	cudaError_t LaunchVertexAttributes(const DeviceProgram& prog, const float* vertices, uint32_t vertex_count,
		float* normals, uint8_t* colors, cudaStream_t stream, VertexOrder order = VertexOrder());
}

namespace tg
{
	// ---- Sodapop's meshing job (tg_sodapop.cu) ---------------------------------------
	// NaiveSurfaceNetsScratch's lattice (sodapop.cpp:150-177): cell (i, j, k), i < SX,
	// j < SY, is number i + j*SX + k*SX*SY and has corners at G + (i..i+1, ...) * D per
	// axis.  The point cache holds numbers below Limit (a multiple of its 64-entry buckets),
	// which reaches one layer past SZ; the lattice has (SX+1) x (SY+1) x LZ points.
	struct SodapopGrid
	{
		float G[3];
		float D[3];
		int64_t SX, SY, SZ;
		int64_t Limit;
		int64_t LZ;
	};

	// clamp(SDFOctree::Eval(p, Exact = false), -100, 100) at every lattice point (x fastest).
	cudaError_t LaunchSodapopLattice(const DeviceProgram& prog, const SodapopGrid& g, float* lattice, cudaStream_t stream);
	// Point cache: cached[n] = 1 for every cell number n < Limit inside one of the leaf
	// boxes (6 int64 per leaf: x0 x1 y0 y1 z0 z1, inclusive; n = x + y*SX + z*SX*SY).
	cudaError_t LaunchSodapopCache(const int64_t* boxes, int leaves, const SodapopGrid& g, uint8_t* cached, cudaStream_t stream);
	// One bit per cell number below Limit: cached and its corners not all of one sign.
	cudaError_t LaunchSodapopFlags(const float* lattice, const uint8_t* cached, const SodapopGrid& g, uint32_t* words,
		cudaStream_t stream);
	// Vertex, cell number and triangle count of every flagged cell, at its rank.
	cudaError_t LaunchSodapopVertices(const float* lattice, const SodapopGrid& g, const uint32_t* words, const uint32_t* word_base,
		float* positions, uint32_t* cells, uint32_t* face_counts, cudaStream_t stream);
	cudaError_t LaunchSodapopFaces(const float* lattice, const SodapopGrid& g, const uint32_t* words, const uint32_t* word_base,
		const uint32_t* cells, const uint32_t* face_base, uint32_t vertex_count, uint32_t* faces, cudaStream_t stream);
	// Gradient normal and shaded colour (4 floats) per vertex.
	cudaError_t LaunchSodapopAttributes(const DeviceProgram& prog, const float* positions, uint32_t vertex_count, float* normals,
		float* colors, cudaStream_t stream);
}

namespace tg
{
	// ---- point-cloud and MagicaVoxel exports (tg_exports.cu) --------------------------
	// PointCloudExportThread's lattice (export.cpp:384-400): IX*IY*IZ voxels from Start at
	// Step per axis (IX = ceil((max - min) / step) per axis), centres offset by Half.
	struct CloudSpec
	{
		float Start[3];
		float Step[3];
		float Half[3];          // Step / 2
		float Diagonal;         // length(Half)
		int32_t IX, IY, IZ;
		int64_t Total;          // IX * IY * IZ (< 2^31, the reference's int)
	};
	// VoxExport's lattice (magica.cpp:29-40): SX*SY*SZ voxels over the tree bounds.
	struct VoxSpec
	{
		float Min[3], Max[3];
		int32_t SX, SY, SZ;
		float Radius;
		int64_t Total;
	};

	// Both voxel tests first decide 8^3-voxel bricks with one bound each (bits in
	// `brick_bits`, VoxelBrickWords of scratch), then test the voxels of the rest.
	size_t VoxelBrickWords(int sx, int sy, int sz);
	// One bit per voxel (cell number order): |octree distance at the centre| < Diagonal.
	cudaError_t LaunchCloudFlags(const DeviceProgram& prog, const CloudSpec& s, uint32_t* brick_bits, uint32_t* words, cudaStream_t stream);
	// Refined point of each listed cell (*count of them, at most `capacity`).
	cudaError_t LaunchCloudRefine(const DeviceProgram& prog, const CloudSpec& s, const uint32_t* cells, const uint32_t* count,
		uint32_t capacity, int iterations, float* points, cudaStream_t stream);
	// One bit per voxel: |full-tree distance at the centre| <= Radius.
	cudaError_t LaunchVoxFlags(const DeviceProgram& prog, const VoxSpec& s, uint32_t* brick_bits, uint32_t* words, cudaStream_t stream);
}

namespace tg
{
	// ---- learned distance bound (tg_field.cu) ----------------------------------------
	// A multiresolution hash grid (16 levels x 2 features) feeds a 32 -> 64 -> 64 -> 64 -> 1
	// ReLU network whose three hidden layers run as BF16 x BF16 -> FP32 tcgen05 matrix
	// multiplies; the output layer is an FP32 dot product.
	constexpr int kFieldLevels = 16;
	constexpr int kFieldInputs = 2 * kFieldLevels;
	constexpr int kFieldHidden = 64;

	struct FieldGrid
	{
		float Lo[3];                 // domain box corner
		float Scale[3];              // 1 / domain extent per axis
		int Res[kFieldLevels];       // cells per axis at each level
		uint32_t DenseLevels;        // bit l: level l indexed densely, (Res + 1)^3 <= TableSize
		uint32_t TableSize;          // entries per level, a power of two
		float Clamp;                 // the network approximates clamp(d, -Clamp, Clamp)
	};

	// Offsets (floats) in the network's FP32 parameter vector; weights are [out][in].
	enum : int
	{
		kFieldW1 = 0, kFieldB1 = 2048, kFieldW2 = 2112, kFieldB2 = 6208, kFieldW3 = 6272, kFieldB3 = 10368,
		kFieldW4 = 10432, kFieldB4 = 10496, kFieldParams = 10497
	};

	// Device image of the network the kernels stage into shared memory with one bulk copy:
	// W1, W2, W3 as BF16 tiles in the tensor-core operand layout, then FP32 b1, b2, b3,
	// W4 (rounded to BF16) and b4.
	constexpr uint32_t kImageW1 = 0, kImageW2 = 4096, kImageW3 = 12288, kImageTail = 20480, kImageBytes = 21520;

	struct AdamStep
	{
		float Rate, Beta1, Beta2, Epsilon;
		float Correction1, Correction2;    // 1 - beta^t
	};

	cudaError_t LaunchFieldPack(const float* mlp, uint8_t* image, cudaStream_t stream);
	// Network output at n points (x, y, z at points + i * stride).  status: set nonzero
	// after a timed-out wait.
	cudaError_t LaunchFieldEval(const FieldGrid& grid, const float2* table, const uint8_t* image, const float* points, int64_t n,
		int stride, float* out, int* status, cudaStream_t stream);
	// Adds d(loss)/d(parameters) for the mean squared error over n samples (x, y, z, d)
	// against clamp(d) to table_grad / mlp_grad and the summed squared error to *loss.
	cudaError_t LaunchFieldTrain(const FieldGrid& grid, const float2* table, const uint8_t* image, const float4* samples, int64_t n,
		float2* table_grad, float* mlp_grad, float* loss, int* status, cudaStream_t stream);
	// Adam on n parameters; zeroes the gradient it consumes.
	cudaError_t LaunchAdam(float* params, float* grads, float* m, float* v, int64_t n, const AdamStep& step, cudaStream_t stream);
	// Uniform points in [lo, hi) from a counter-based generator: sample i goes to
	// out[i * stride + offset] with w = 0.
	cudaError_t LaunchFieldUniform(uint64_t seed, const float* lo, const float* hi, float4* out, int64_t n, int64_t stride,
		int64_t offset, cudaStream_t stream);
	// w = the whole tree's distance (SDFNode::Eval) at each sample.
	cudaError_t LaunchEvalFull(const DeviceProgram& prog, float4* samples, int64_t n, cudaStream_t stream);
	// Bit i of words: |w_i| < band.
	cudaError_t LaunchBandFlags(const float4* samples, int64_t n, float band, uint32_t* words, cudaStream_t stream);
	// Flagged samples in order: the one of rank r goes to out[(first + r) * stride + offset]
	// while first + r < limit.
	cudaError_t LaunchBandCompact(const float4* samples, int64_t n, const uint32_t* words, const uint32_t* word_base,
		float4* out, int64_t first, int64_t limit, int64_t stride, int64_t offset, cudaStream_t stream);
	// Brick culling with the network: a brick's bit is set unless |net(centre)| exceeds its
	// ball's radius plus `margin` or it misses the root cube (as LaunchClassifyBricks).
	cudaError_t LaunchFieldClassifyBricks(const DeviceProgram& prog, const GridSpec& g, int B, const FieldGrid& grid,
		const float2* table, const uint8_t* image, float margin, uint32_t* brick_bits, int* status, cudaStream_t stream);
	// Sphere tracing with network steps and exact final steps (see tg_field.cu); counters
	// (optional) accumulate network iterations and exact steps.
	// travel/state: per-ray scratch (count*width*height each) between the two kernels.
	cudaError_t LaunchRenderField(const DeviceProgram& prog, const CameraBasis* cameras, int count, int width, int height, int steps,
		float epsilon, const FieldGrid& grid, const float2* table, const uint8_t* image, float margin, float switch_at, float* travel,
		uint32_t* state, float* depth, float* normals, uint8_t* colors, unsigned long long* counters, int* status, cudaStream_t stream);
	// Tensor-core operand-layout check: D = A * B^T through the descriptors the network
	// kernels use.  mode 0: A 128x64 and B 64x64 read K-major; mode 1: A = a^T and
	// B = b^T for a 128x128 and b 128x144 read MN-major (K = 128 rows); mode 2: A 128x64
	// K-major, B = b^T for b 64x64 read MN-major.  Inputs FP32 (rounded to BF16), D 128 x N.
	cudaError_t LaunchDebugMma(int mode, const float* a, const float* b, float* d, int* status, cudaStream_t stream);
}

namespace tg
{
	// ---- many trees in one persistent launch (tg_batch.cu) ---------------------------
	struct BatchModel
	{
		DeviceProgram Prog;
		GridSpec Grid;
		int B, NBX, NBY, NBZ;      // brick edge (cells) and bricks per axis
		int Lanes, HasPaint;       // lattice points per thread; colours wanted
		int64_t Bricks;
		int64_t Lattice;           // first float of the model's lattice in the pool
		int64_t BrickWord0;        // first word of its brick bits
		int64_t CellWord0;         // first word of its cell bits
		int Cull;                  // bricks kept by: 0 the exact test; 1 the model's learned bound
		                           // (its bits written before the launch); 2 the bound, then
		                           // the exact test on the bricks it keeps
	};

	struct BatchState
	{
		const BatchModel* Models;
		int Count;
		int Attributes;
		const int64_t* BrickWord0;     // per model, ascending
		const int64_t* Tile0;          // per model, ascending: first 8 x 4 brick patch of its classification
		int64_t TilesTotal;
		const uint64_t* CellBit0;      // per model: CellWord0 * 32
		const int64_t* CellWords;      // per model
		int64_t BrickWordsTotal, CellWordsTotal;
		uint32_t* BrickBits;
		uint32_t* BrickWordBase;
		uint32_t* BrickList;
		uint32_t* BrickTops;           // per global brick: the kept brick's descent (cell | shared << 31)
		uint32_t* CellBits;
		uint32_t* CellWordBase;
		uint64_t* ActiveCells;
		float* Lattice;
		uint32_t CapVertices, CapFaces;
		float* Vertices;
		float* Normals;
		uint8_t* Colors;
		uint32_t* Cubes;
		uint32_t* FaceCounts;
		uint32_t* FaceBase;
		uint32_t* Faces;
		uint32_t* VertexBase;          // per model + 1: first vertex (global numbering)
		uint32_t* FaceBaseModel;       // per model + 1: first face
		uint32_t* Counters;            // kept bricks, active cells, vertices, faces, overflow bits; [8..15]: cost
		                               // classes' brick counts and cursors
		uint32_t* ScanPartials;        // blocks + 1
		unsigned* Barrier;             // arrival count, generation
		int* Status;                   // 2: a barrier wait ran out; 3: cancelled
		const volatile int* Cancel;    // host-mapped flag polled at every grid barrier (null: none)
		const uint64_t* Knobs;         // barrier limit in ns (0: default), late block + 1, its delay in ns
	};

	size_t BatchSharedBytes(int max_stack);
	int BatchThreads();
	// Co-resident blocks of the cooperative batch kernel on this device.
	cudaError_t BatchMaxBlocks(int max_stack, int* blocks);
	cudaError_t LaunchBatchExport(const BatchState& s, int blocks, int max_stack, cudaStream_t stream);
}
