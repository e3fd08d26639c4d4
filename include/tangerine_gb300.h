/*
 * tangerine_gb300 -- C ABI of the GB300 (sm_103a) CSG evaluation and export-meshing engine.
 *
 * Two layers:
 *
 *  1. Tangerine's own C API for CSG trees (tangerine/c_sdf.cpp:27-180 and the export entry
 *     points tangerine/export.cpp:611-621), which the reference ships disabled (#if 0) and
 *     which its Racket FFI binds (package/tangerine/eval.rkt:39-68, export.rkt:26-28).
 *     Same names, argument order and meaning.  Handles are reference-counted trees: an
 *     operator (Make*Op) takes over the references of its operand handles, as the raw
 *     pointer API did, so a caller discards only the root.  ClipTree returns a new handle.
 *
 *  2. The GPU-native entry points (tg_*): compile a tree into octree cells and record
 *     programs once, then evaluate lattices and export meshes on the GPU.  Every tg_* call
 *     returns a tg_status (0 = success); tg_last_error() describes the last failure on the
 *     calling thread.  Calls on one program are thread-compatible, not thread-safe.
 *
 * All pointers are plain host pointers unless a parameter says "device".  `stream` is a
 * cudaStream_t (NULL: the library's own stream); calls return after their work on that
 * stream has finished.
 */
#ifndef TANGERINE_GB300_H
#define TANGERINE_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define TANGERINE_API __declspec(dllexport)
#else
#define TANGERINE_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Tangerine's C API (tangerine/c_sdf.cpp) ----------------------------------------- */

/* SDFNode::RayMarch result (tangerine/sdf_evaluator.h:75-80). */
typedef struct RayHit
{
	bool Hit;
	float Travel;
	float Position[3];
} RayHit;

/* EvalTree: SDFNode::Eval at one point (c_sdf.cpp:30-34). */
TANGERINE_API float EvalTree(void* Handle, float X, float Y, float Z);
/* ClipTree: the subtree that can matter within Radius of the point; NULL when nothing
 * does, or when the clipped tree's distance there exceeds Radius (c_sdf.cpp:38-53). */
TANGERINE_API void* ClipTree(void* Handle, float X, float Y, float Z, float Radius);
/* RayMarchTree: sphere tracing on the full tree (c_sdf.cpp:56-66). */
TANGERINE_API RayHit RayMarchTree(void* Handle, float RayStartX, float RayStartY, float RayStartZ,
                                  float RayDirX, float RayDirY, float RayDirZ, int MaxIterations, float Epsilon);
/* DiscardTree: drop this handle's reference (c_sdf.cpp:70-74). */
TANGERINE_API void DiscardTree(void* Handle);
/* TreeHasFiniteBounds (c_sdf.cpp:77-80). */
TANGERINE_API bool TreeHasFiniteBounds(void* Handle);
/* MoveTree / RotateTree (quat(W, X, Y, Z)) / AlignTree (c_sdf.cpp:86-106). */
TANGERINE_API void MoveTree(void* Handle, float X, float Y, float Z);
TANGERINE_API void RotateTree(void* Handle, float X, float Y, float Z, float W);
TANGERINE_API void AlignTree(void* Handle, float X, float Y, float Z);
/* PaintTree: a new sRGB material on every unpainted brush (c_sdf.cpp:110-114). */
TANGERINE_API void PaintTree(float Red, float Green, float Blue, void* Handle);
/* Brushes (c_sdf.cpp:118-146): half-extents and radii as SDF:: takes them. */
TANGERINE_API void* MakeSphereBrush(float Radius);
TANGERINE_API void* MakeEllipsoidBrush(float RadipodeX, float RadipodeY, float RadipodeZ);
TANGERINE_API void* MakeBoxBrush(float ExtentX, float ExtentY, float ExtentZ);
TANGERINE_API void* MakeTorusBrush(float MajorRadius, float MinorRadius);
TANGERINE_API void* MakeCylinderBrush(float Radius, float Extent);
TANGERINE_API void* MakePlaneOperand(float NormalX, float NormalY, float NormalZ);
/* Set operators (c_sdf.cpp:150-178); they take over the operand handles. */
TANGERINE_API void* MakeUnionOp(void* LHS, void* RHS);
TANGERINE_API void* MakeDiffOp(void* LHS, void* RHS);
TANGERINE_API void* MakeInterOp(void* LHS, void* RHS);
TANGERINE_API void* MakeBlendUnionOp(float Threshold, void* LHS, void* RHS);
TANGERINE_API void* MakeBlendDiffOp(float Threshold, void* LHS, void* RHS);
TANGERINE_API void* MakeBlendInterOp(float Threshold, void* LHS, void* RHS);

/* The rest of SDF:: (tangerine/sdf_evaluator.h:223-264) that c_sdf.cpp never exposed. */
TANGERINE_API void* MakeConeBrush(float Radius, float Height);
TANGERINE_API void* MakeConinderBrush(float RadiusL, float RadiusH, float Height);
TANGERINE_API void* MakeFlateOp(void* Handle, float Radius);
TANGERINE_API void* MakeStencilOp(void* Handle, void* Mask, float Red, float Green, float Blue, bool ApplyToNegative);
TANGERINE_API void ScaleTree(void* Handle, float Scale);
/* Replays a tree spec: the postfix construction word stream tangerine_gb300.workloads
 * writes (op codes there).  NULL on a malformed spec (tg_last_error explains). */
TANGERINE_API void* BuildTreeFromSpec(const float* Spec, int Count);
/* The spec that rebuilds this tree exactly (BuildTreeFromSpec): brushes with their whole
 * transforms and materials, operators in their stored order.  Returns the word count
 * (-1: null handle) and copies at most `capacity` words. */
TANGERINE_API int64_t tg_tree_spec(void* Handle, float* Out, int64_t Capacity);
/* Used by the Lua tangerine.sdf surface (tangerine/lua_sdf.cpp), which never mutates a tree
 * in place: SDFNode::Copy (a new handle); paint_over (ApplyMaterial with Force); and
 * SDF::RotateX/Y/Z (degrees, through sinf / cosf as the reference). */
TANGERINE_API void* CopyTree(void* Handle);
/* SDFNode::Gradient on the host (Lua's gradient, lua_sdf.cpp:398-405): 3 floats to Out. */
TANGERINE_API void GradientTree(void* Handle, float X, float Y, float Z, float* Out);
TANGERINE_API void PaintOverTree(float Red, float Green, float Blue, void* Handle);
TANGERINE_API void RotateTreeX(void* Handle, float Degrees);
TANGERINE_API void RotateTreeY(void* Handle, float Degrees);
TANGERINE_API void RotateTreeZ(void* Handle, float Degrees);

/* Export the tree's bounds at 1/GridSize spacing to a file, synchronously
 * (ExportCommon + MeshExportThread, tangerine/export.cpp:320-381, 595-621).
 * RefineIterations is accepted and unused, as in the reference mesh export. */
TANGERINE_API void ExportSTL(void* Handle, float GridSize, int RefineIterations, const char* Path);
TANGERINE_API void ExportPLY(void* Handle, float GridSize, int RefineIterations, const char* Path);

/* ---- GPU-native API ----------------------------------------------------------------- */

typedef int tg_status;
enum
{
	TG_OK = 0,
	TG_ERR_INVALID = 1,      /* bad argument */
	TG_ERR_UNBOUNDED = 2,    /* tree has infinite or empty bounds */
	TG_ERR_CUDA = 3,         /* CUDA runtime error (no GPU, launch failure, ...) */
	TG_ERR_MEMORY = 4,       /* host or device allocation failed */
	TG_ERR_IO = 5,           /* file could not be written */
	TG_ERR_UNSUPPORTED = 6,  /* input outside what the kernels handle */
	TG_ERR_CANCELLED = 7,    /* stopped by CancelExport(true) or tg_batch_cancel */
	TG_ERR_BUSY = 8,         /* an asynchronous export is still running */
};

typedef struct tg_program tg_program;

/* Lattice of sample points x0 + i*step (i < nx), y0 + j*step_y, z0 + k*step_z; x varies
 * fastest.  step_y / step_z of 0 mean `step` (one step for every axis). */
typedef struct tg_grid
{
	float x0, y0, z0;
	float step;
	int64_t nx, ny, nz;
	float step_y, step_z;
} tg_grid;

typedef struct tg_program_info
{
	int32_t octree_cells;
	int32_t code_quads;
	int32_t materials;
	int32_t has_paint;          /* colours are exported */
	int32_t max_stack;
	float bounds_min[3], bounds_max[3];
	double compile_seconds;
	int64_t distance_quads;     /* summed over all cells */
} tg_program_info;

/* A mesh in host memory (library-allocated, page-locked when possible; release with
 * tg_mesh_free, which recycles the blocks for later exports).  Vertex v is the
 * vertex of active cube cubes[v] (x + y*sx + z*sx*sy); faces are vertex index triples. */
typedef struct tg_mesh
{
	uint64_t vertex_count;
	uint64_t face_count;
	float* vertices;            /* 3 per vertex */
	float* normals;             /* 3 per vertex */
	uint8_t* colors;            /* 3 per vertex, NULL when the tree has no paint */
	uint32_t* faces;            /* 3 per face */
	uint32_t* cubes;            /* 1 per vertex */
} tg_mesh;

/* The same mesh left in device memory owned by the library (valid until the next export
 * call on this thread's engine). */
typedef struct tg_device_mesh
{
	uint64_t vertex_count;
	uint64_t face_count;
	const float* vertices;      /* device */
	const float* normals;       /* device */
	const uint8_t* colors;      /* device, NULL without paint */
	const uint32_t* faces;      /* device */
	const uint32_t* cubes;      /* device */
} tg_device_mesh;

enum
{
	TG_MESH_ATTRIBUTES = 1u,    /* compute gradient normals and colours */
	TG_MESH_DENSE = 2u,         /* evaluate every lattice point, as the reference does; by
	                               default bricks that provably hold no surface are skipped
	                               (same mesh, bit for bit) */
	/* bits 8..15: brick edge in cells for the culled export (1..32; 0 = 7)
	   bits 16..19: lattice points per thread sharing one pass over the records (1, 2, 4;
	   0 = 2 culled, 4 dense) */
};

/* Builds the export octree (target size 0.25, coalescing) and compiles every cell's
 * clipped subtree; uploads them to the current device. */
TANGERINE_API tg_status tg_compile(void* tree, tg_program** out);
TANGERINE_API void tg_program_free(tg_program* program);
TANGERINE_API tg_status tg_program_get_info(const tg_program* program, tg_program_info* out);
/* Distance program words of the whole tree exactly as Tangerine's SDFInterpreter holds
 * them (for checking).  Returns the word count; copies at most `capacity`. */
TANGERINE_API int64_t tg_tree_reference_words(void* tree, uint32_t* out, int64_t capacity);

/* Host-only check of the export octree (no GPU needed): the cells depth-first, 14 floats
 * each (pivot xyz, bounds min xyz, max xyz, terminus, has evaluator, first word, word
 * count, stack size), 8 child indices each (-1: none), and every cell's distance program
 * words concatenated.  Returns the cell count (-1 when SDFOctree::Create would fail);
 * copies at most the given capacities. */
TANGERINE_API int64_t tg_debug_octree(void* tree, float* cells, int32_t* children, int64_t cell_capacity,
                                      uint32_t* words, int64_t word_capacity, int64_t* word_count);

/* The same dump of Sodapop's meshing octree (see tg_sodapop_mesh). */
TANGERINE_API int64_t tg_debug_meshing_octree(void* tree, float* cells, int32_t* children, int64_t cell_capacity,
                                              uint32_t* words, int64_t word_capacity, int64_t* word_count);
/* Host-only: builds and compiles the export (or meshing) octree without uploading it and
 * reports the seconds spent in the octree and in all of the compile. */
TANGERINE_API tg_status tg_debug_compile_seconds(void* tree, int meshing, double* octree_seconds, double* total_seconds);
/* Host-only check of the early brick test's input: compiles the export octree with the
 * root-cell hook tg_export_tree uses and checks that the root program it handed out (before
 * the levels below the root existed) has node 0's pivot and clip radius and, record for
 * record, node 0's distance program.  TG_OK with the program's quads (stop included) and
 * stack depth; TG_ERR_INVALID with the difference in tg_last_error otherwise. */
TANGERINE_API tg_status tg_debug_root_program_check(void* tree, int64_t* code_quads, int32_t* stack_size);
/* Host-only check of tg_export_tree's deferred surface programs: the export tree compiled
 * whole and compiled with its surface programs left out, then emitted into a separate
 * image as the export does into its staging buffer, must give the same program image,
 * node table and header bit for bit.  TG_OK, or TG_ERR_INVALID with the difference. */
TANGERINE_API tg_status tg_debug_deferred_surfaces_check(void* tree);
/* Host-only plan of tg_sodapop_mesh: grid gets origin xyz, step xyz, cells xyz, the point
 * cache's limit and the lattice's z layers (11 floats); boxes the leaves' inclusive integer
 * point-cache spans (6 per leaf, up to box_capacity leaves); leaves the leaf count. */
TANGERINE_API tg_status tg_debug_sodapop_plan(void* tree, float density, float* grid, int64_t* boxes, int64_t box_capacity,
                                              int64_t* leaves);

/* The lattice MeshExportThread builds for (min, max, step): min moves down two steps;
 * ceil((max - min) / step) cells, one more lattice point, per axis (export.cpp:324-337). */
TANGERINE_API tg_status tg_export_grid(const float model_min[3], const float model_max[3], float step, tg_grid* out);
/* The same with a step per axis, as MeshExportThread's vec3 Step. */
TANGERINE_API tg_status tg_export_grid_axes(const float model_min[3], const float model_max[3], const float step[3],
                                            tg_grid* out);

/* SDFOctree::Eval(p, Exact = true) at every lattice point.  `out` holds nx*ny*nz floats,
 * host memory, or device memory when out_is_device is nonzero. */
TANGERINE_API tg_status tg_eval_grid(tg_program* program, const tg_grid* grid, float* out, int out_is_device, void* stream);

/* Octree distances at n arbitrary points (host arrays, 3 floats per point). */
TANGERINE_API tg_status tg_eval_points(tg_program* program, const float* points, int64_t n, float* out, void* stream);

/* Naive surface nets over the lattice (cells between lattice points), then gradient
 * normals and colours per vertex.  Results in host memory. */
TANGERINE_API tg_status tg_export_mesh(tg_program* program, const tg_grid* grid, uint32_t flags, tg_mesh* out, void* stream);
/* Same, results left on the device. */
TANGERINE_API tg_status tg_export_mesh_device(tg_program* program, const tg_grid* grid, uint32_t flags, tg_device_mesh* out, void* stream);
TANGERINE_API void tg_mesh_free(tg_mesh* mesh);

/* tg_export_mesh for callers that must not allocate GPU memory once running (an
 * application that gives all device memory to its own pool at start-up, or a thread that
 * cannot absorb cudaMalloc's device-wide synchronisation).  No counterpart in the
 * reference: Tangerine's export runs on the CPU and allocates freely.
 *
 * The results equal tg_export_mesh's bit for bit, but this path always runs the dense
 * kernels: every lattice point is evaluated, as the reference does, with no brick culling
 * (at 128^3 that is several times the culled export's device time).  Nothing is allocated:
 * the outputs are the caller's device buffers (vertices and normals 3 floats per vertex,
 * colors 3 bytes per vertex, faces 3 uint32 per face, cubes 1 uint32 per vertex) and the
 * scratch (lattice, active-cell bitmask, prefix sums) lives in one fixed 64 MiB device
 * array inside the library -- about a 240^3 lattice at most.
 *  - flags: TG_MESH_ATTRIBUTES (normals and colours) and TG_MESH_DENSE (a no-op here); any
 *    other bit fails with TG_ERR_UNSUPPORTED.  `normals` may be NULL without
 *    TG_MESH_ATTRIBUTES, `colors` when the tree has no paint.
 *  - Larger lattices fail with TG_ERR_UNSUPPORTED.  Too small a vertex capacity fails with
 *    TG_ERR_INVALID and counts[0] = the vertices needed (counts[1] stays 0: the face count
 *    is known only once the vertices fit); too small a face capacity fails with
 *    TG_ERR_INVALID and counts[1] = the faces needed.
 *  - The array is part of a CUDA module that loads lazily: a device reserves the 64 MiB
 *    the first time this function runs on it, and holds them until the process exits.
 *    Calling it with every pointer NULL only does that set-up on the current device
 *    (looks up the array's address with cudaGetSymbolAddress and caches it).  Make that
 *    first call before giving the rest of device memory to a pool, and before any stream
 *    capture.  cudaDeviceReset is not supported while the library is in use (the cached
 *    address would be stale).
 *  - All calls share the array, which keeps the last call's contents.  Calls that overlap
 *    on the GPU (several threads or streams at once) race on it: serialise them.
 *  - stream NULL is the legacy default stream here (the other entry points take NULL as
 *    the library's own stream). */
TANGERINE_API tg_status tg_export_mesh_noalloc(tg_program* program, const tg_grid* grid, uint32_t flags,
                                               float* vertices, float* normals, uint8_t* colors, uint32_t* faces,
                                               uint32_t* cubes, uint64_t vertex_capacity, uint64_t face_capacity,
                                               uint64_t* counts, void* stream);

/* Whole reference export path from a tree: octree + compile, lattice, surface nets,
 * normals, colours, copy back to the host (MeshExportThread minus the file write).  The
 * fastest form for a tree exported once: the GPU tests the bricks on the root cell's
 * program while the host builds the rest of the octree, and the surface programs are
 * emitted while the GPU runs the first export stages; the mesh is the one tg_compile +
 * tg_export_mesh give, bit for bit.  Holds the library's engine for the whole call. */
TANGERINE_API tg_status tg_export_tree(void* tree, const float model_min[3], const float model_max[3], float step,
                                       tg_mesh* out, void* stream);

/* Sodapop's meshing job for one drawable (MeshingJob::NaiveSurfaceNets,
 * tangerine/sodapop.cpp:562-897), on the GPU:
 *  - the meshing octree: SDFOctree::Create(.25, false, 3), then every incomplete cell
 *    populated with Populate(false, 3, -1);
 *  - a lattice over the root's bounds at floor(density) samples per unit (at least 8 per
 *    axis), one step per axis, two extra steps below the minimum and three extra cells
 *    (sodapop.cpp:153-177); Sodapop::Populate uses density 20 plus the caller's push;
 *  - clamp(octree distance with the non-exact descent, -100, 100) at its points;
 *  - surface nets over the cells inside the octree leaves' aligned boxes (the point
 *    cache), vertices in cell-number order;
 *  - per vertex the gradient normal and the colour MaterialPBRBR gives with V = N (white
 *    where no material applies), alpha 1.
 * The reference then permutes the vertices (ApplyVertexSequence) for its renderer; that
 * order depends on thread timing and is not reproduced.  Results in host memory; release
 * with tg_drawable_free. */
typedef struct tg_drawable
{
	uint64_t vertex_count;
	uint64_t face_count;
	float* positions;           /* 3 per vertex */
	float* normals;             /* 3 per vertex */
	float* colors;              /* 4 per vertex (RGBA) */
	uint32_t* faces;            /* 3 per face */
	uint32_t* cells;            /* 1 per vertex: x + y*sx + z*sx*sy */
	float grid_origin[3];       /* lattice point (0, 0, 0) */
	float grid_step[3];
	int64_t grid_cells[3];      /* sx, sy, sz */
	double compile_seconds;     /* meshing octree + programs, on the host */
	double gpu_seconds;         /* upload, kernels and copies */
} tg_drawable;

TANGERINE_API tg_status tg_sodapop_mesh(void* tree, float density, tg_drawable* out, void* stream);
TANGERINE_API void tg_drawable_free(tg_drawable* drawable);
/* MeshExport(Path, UseBaseColor = true, Format, Scale) (export.cpp:495-563): the drawables of
 * placed models written as one STL (format 0) or PLY (1) file.  frames: 8 floats per
 * drawable, the model's LocalToWorld (rotation w x y z, translation, scale), or NULL for
 * none; positions go through its matrix and are multiplied by scale, normals are written as
 * they are, colours as bytes 0xFF * c, faces offset by the vertices before.  The STL facet
 * normal is the normalised sum of its corners' normals. */
TANGERINE_API tg_status tg_write_drawables(const tg_drawable* drawables, const float* frames, int count, const char* path,
                                           int format, float scale);

/* PointCloudExportThread (export.cpp:384-480) on the GPU: the centres of the voxels of the
 * ceil((max - min) / step) lattice from model_min whose octree distance is below the
 * half-voxel diagonal, moved by refine_iterations steps of -distance along the gradient,
 * clamped to the voxel and kept only when they stay within the diagonal; with
 * TG_MESH_ATTRIBUTES, gradient normals and colour bytes as WritePLY(Octree, ...) takes them.
 * The reference's threads push points in a run-dependent order; here they come in voxel
 * order.  Results as a tg_mesh without faces (cubes = each point's voxel number, x
 * fastest); release with tg_mesh_free. */
TANGERINE_API tg_status tg_export_point_cloud(tg_program* program, const float model_min[3], const float model_max[3],
                                              const float step[3], int refine_iterations, uint32_t flags, tg_mesh* out,
                                              void* stream);

/* VoxExport's voxels (magica.cpp:27-72) on the GPU: the ivec3(ceil(max - min) * grid_size)
 * lattice over the tree bounds, a voxel kept when |SDFNode::Eval| at its centre
 * mix(min, max, (i + .5) / size) is at most the half-voxel radius; colour index
 * abs(color_index) % 255 + 1.  Voxels in voxel order (x fastest). */
typedef struct tg_voxels
{
	uint64_t count;
	int32_t* voxels;            /* 4 per voxel: x, y, z, colour index */
	int32_t size[3];
	float radius;
} tg_voxels;

TANGERINE_API tg_status tg_export_voxels(tg_program* program, float grid_size, int color_index, tg_voxels* out, void* stream);
TANGERINE_API void tg_voxels_free(tg_voxels* voxels);
/* The MagicaVoxel file VoxWriter writes for these voxels added in order (version 150, one
 * model per 126-voxel cube, a transform per cube, no palette). */
TANGERINE_API tg_status tg_write_vox(const tg_voxels* voxels, const char* path);
/* ExportMagicaVoxel (magica.cpp:79-83, shipped disabled): voxelise the tree and write the
 * file, synchronously. */
TANGERINE_API void ExportMagicaVoxel(void* Handle, float GridSize, int ColorIndex, const char* Path);
/* MeshExport (export.h:37, export.cpp:566-580): starts the export on a detached host
 * thread and returns at once, as the reference does.  Format 0 = STL, 1 = PLY, as
 * ExportFormat; ExportPointCloud selects the point-cloud export (PLY only, as the reference
 * writes nothing else for it).  Vertices are multiplied by Scale when written.  Step is
 * per axis; RefineIterations applies to point clouds only, as in the reference.
 * Arguments are checked before the thread starts (a bad format returns TG_ERR_UNSUPPORTED
 * and starts nothing); one export runs at a time (TG_ERR_BUSY while one is running).  The
 * job's own outcome comes from tg_export_result; its progress from GetExportProgress. */
TANGERINE_API tg_status MeshExport(void* Handle, const char* Path, const float ModelMin[3], const float ModelMax[3],
                                   const float Step[3], int RefineIterations, int Format, bool ExportPointCloud, float Scale);

/* ExportProgress (export.h:27-34), as GetExportProgress (export.cpp:483-492) fills it.
 * Stage: 0 idle or finished, 1 generation (octree, lattice and surface nets, or the
 * point cloud's voxel search), 2 refinement (point clouds), 3 vertex attributes and the
 * file write.  Each fraction runs from 0 to 1 over its stage; the GPU finishes a stage in
 * milliseconds, so they advance by whole phases (the reference counts single cells). */
typedef struct ExportProgress
{
	int Stage;
	float Generation;
	float Refinement;
	float Secondary;
	float Write;
} ExportProgress;

TANGERINE_API ExportProgress GetExportProgress(void);
/* CancelExport (export.cpp:582-592).  Halt = true stops the running export at its next
 * phase boundary: no file is written (a partly written file is removed) and the job ends
 * with TG_ERR_CANCELLED.  The reference instead goes on to write whatever part of the mesh
 * it had.  Halt = false is the reference's "good enough": it ends the current stage early
 * -- for a point cloud, the refinement is skipped when pressed before or during it; a mesh
 * export has no partial stage result and goes on. */
TANGERINE_API void CancelExport(bool Halt);
/* Outcome of the last MeshExport job: with wait != 0, blocks until it has finished; with
 * wait == 0, TG_ERR_BUSY while it runs.  TG_OK when no job ran.  On failure the job's
 * message becomes this thread's tg_last_error. */
TANGERINE_API tg_status tg_export_result(int wait);

/* SDFNode::RayMarch (sdf_evaluator.cpp:336-353) on the whole tree for n rays, on the GPU:
 * the reference's step sequence, so hit flags, travel (+inf on a miss) and end positions
 * match it bit for bit.  Host arrays, 3 floats per origin / direction / position. */
TANGERINE_API tg_status tg_ray_march(tg_program* program, const float* origins, const float* dirs, int64_t n,
                                     int max_iterations, float epsilon, uint8_t* hit, float* travel, float* position,
                                     void* stream);

/* The app's other ray casts, batched: mode 0 is tg_ray_march; mode 1 is Lua's magnet cast
 * (lua_sdf.cpp:410-437), whose `dirs` are target points: the direction is
 * normalize(target - origin); mode 2 is SDFModel::RayMarch (sdf_model.cpp:261-266), mouse
 * picking on a placed model: frame = the model's rotation quaternion (w, x, y, z),
 * translation (x, y, z) and scale; the ray goes into the model's frame and marches 1000
 * iterations at epsilon 0.001, whatever `iterations` and `epsilon` say, as the reference
 * ignores its own arguments there.  Positions are in the frame the march ran in. */
TANGERINE_API tg_status tg_ray_query(tg_program* program, int mode, const float frame[8], const float* origins, const float* dirs,
                                     int64_t n, int iterations, float epsilon, uint8_t* hit, float* travel, float* position,
                                     void* stream);
/* SDFNode::Eval / SDFNode::Gradient on the whole tree at n points, on the GPU: Lua's eval
 * and gradient (lua_sdf.cpp:386-405) and EvalTree, batched.  out: 1 / 3 floats per point. */
TANGERINE_API tg_status tg_eval_tree_points(tg_program* program, const float* points, int64_t n, float* out, void* stream);
TANGERINE_API tg_status tg_gradient_tree_points(tg_program* program, const float* points, int64_t n, float* out, void* stream);

/* Pinhole camera looking from `position` at `target`; `up` fixes the roll; tan_half_fov is
 * tan(vertical field of view / 2).  Pixel (x, y) of a W x H image looks along
 * forward + right*u + up'*v, u = (2(x+0.5)/W - 1) * tan_half_fov * W/H,
 * v = (1 - 2(y+0.5)/H) * tan_half_fov, with forward = normalize(target - position),
 * right = normalize(cross(forward, up)), up' = cross(right, forward). */
typedef struct tg_camera
{
	float position[3];
	float target[3];
	float up[3];
	float tan_half_fov;
} tg_camera;

enum
{
	TG_RENDER_EXACT = 1u,       /* every step on the whole tree, as SDFNode::RayMarch; else
	                               octree-bounded steps (same hits, fewer operations) */
};

/* Sphere-traced depth (travel along the normalised ray, +inf on a miss), gradient normal
 * (0 on a miss) and colour bytes (0 on a miss) for `count` cameras, image after image,
 * rows top to bottom.  depth: count*W*H floats, normals: 3 per pixel, colors: 3 per pixel
 * or NULL.  Host buffers, or device buffers when out_is_device is nonzero. */
TANGERINE_API tg_status tg_render(tg_program* program, const tg_camera* cameras, int count, int width, int height,
                                  int max_steps, float epsilon, uint32_t flags, float* depth, float* normals,
                                  uint8_t* colors, int out_is_device, void* stream);

/* Files in the reference's byte layout (WritePLY / WriteSTL, export.cpp:60-317).
 * The STL writer needs the program for its per-face gradient normals. */
TANGERINE_API tg_status tg_write_ply(const tg_mesh* mesh, const char* path, float scale);
TANGERINE_API tg_status tg_write_stl(tg_program* program, const tg_mesh* mesh, const char* path, float scale, void* stream);

/* Bricks in the last culled export on this process's engine and how many were evaluated. */
TANGERINE_API tg_status tg_last_export_stats(int64_t* bricks, int64_t* active_bricks);

/* The bricks the last culled export evaluated (brick index = bx + nbx * (by + nby * bz),
 * bricks of brick_size^3 cells from the lattice origin), in index order; returns how many
 * there were and copies at most `capacity`. */
TANGERINE_API int64_t tg_last_export_bricks(uint32_t* out, int64_t capacity, int* brick_size);

/* Host wall time of the phases of the last tg_export_tree on this thread: octree build +
 * compile, upload, GPU export, copy back. */
TANGERINE_API tg_status tg_last_export_timing(double* compile_s, double* upload_s, double* gpu_s, double* copy_s);

/* Per-kernel device time of the export pipeline, accumulated while enabled (CUDA events
 * on the launching stream).  Names: "eval_grid", "cell_flags", "scan", "cell_vertices",
 * "faces", "attributes", "face_normals", "eval_points", "classify_bricks", "eval_bricks",
 * "ray_march", "render". */
TANGERINE_API void tg_profile_enable(int enable);
TANGERINE_API int tg_profile_read(const char* kernel, double* total_ms, int64_t* launches);
TANGERINE_API void tg_profile_reset(void);

/* Measures this GPU's FP32 fused-multiply-add throughput in TFLOP/s (2 flops per FMA):
 * the compute roofline of the distance interpreter. */
TANGERINE_API tg_status tg_measure_fp32_peak(double* tflops, void* stream);

/* ---- many trees in one launch ----------------------------------------------------------
 * No counterpart in the reference (which exports one tree per call on a detached thread).
 * The programs' exports run together as one persistent cooperative kernel over a global
 * (model, brick) work queue -- classify, evaluate, surface nets, normals, colours -- replayed
 * from a CUDA graph.  Each model's mesh equals tg_export_mesh's for its program and lattice.
 * The programs must outlive the batch. */
typedef struct tg_batch tg_batch;

typedef struct tg_batch_info
{
	int64_t models, samples;                   /* lattice points over all models */
	int64_t bricks, bricks_evaluated;
	int64_t vertices, faces;
	int graph;                                 /* 1: replayed from a CUDA graph; -1: capture refused, launched directly */
	int blocks;                                /* CTAs of the cooperative launch */
	int reruns;                                /* runs repeated after growing the output buffers */
	double autotune_seconds;
	int64_t device_bytes;
} tg_batch_info;

/* flags: TG_MESH_ATTRIBUTES.  Brick edge 7 and 2 lattice points per thread for every model
 * until tg_batch_autotune or tg_batch_set_tuning. */
TANGERINE_API tg_status tg_batch_create(tg_program* const* programs, const tg_grid* grids, int count, uint32_t flags,
                                        tg_batch** out);
TANGERINE_API void tg_batch_free(tg_batch* batch);
/* Per (lattice extent, program size) class: times single-model exports of one member for
 * brick edges {4, 7, 11, 15} x lattice points per thread {1, 2, 4} and gives the class the
 * fastest. */
TANGERINE_API tg_status tg_batch_autotune(tg_batch* batch, void* stream);
TANGERINE_API tg_status tg_batch_set_tuning(tg_batch* batch, const int* brick_edges, const int* lanes);
TANGERINE_API tg_status tg_batch_get_tuning(const tg_batch* batch, int* brick_edges, int* lanes);
TANGERINE_API tg_status tg_batch_run(tg_batch* batch, void* stream);
/* Cancels a batch run from any thread (cancel = 1), as CancelExport(true) does for the
 * single export: the persistent kernel reads a host-mapped flag at each of its grid
 * barriers, every block leaves after the first barrier that sees it, and tg_batch_run
 * returns TG_ERR_CANCELLED (the outputs are incomplete) and clears the flag.  A cancel that
 * comes after the running batch's last barrier cancels the next run instead; cancel = 0
 * withdraws it. */
TANGERINE_API tg_status tg_batch_cancel(tg_batch* batch, int cancel);
/* Test hook for the persistent kernel's grid barrier: its wait limit (limit_ns; 0 = the
 * default 5 s, else 1 ms..60 s) and one block (late_block; -1 = none) that starts late_ns
 * late (at most 2 s).  With a late start longer than the limit, the other blocks' first
 * wait runs out: every block leaves and tg_batch_run returns TG_ERR_CUDA ("timed out"),
 * the GPU context stays usable, and the next run (knobs back at 0, -1, 0) is whole. */
TANGERINE_API tg_status tg_batch_debug_barrier(tg_batch* batch, uint64_t limit_ns, int late_block, uint64_t late_ns);
/* Test hook for two bounded mbarrier waits.  which = 0: the staged-program copy of the
 * brick evaluation (TG_MESH_STAGED); which = 1: the network-image copy at the start of the
 * surrogate kernels.  With limit_ns > 0 (at most 1 s) the wait is made on an mbarrier that
 * nothing arrives at, so it runs out after limit_ns: the kernel records the failure, waits
 * (bounded) for its own copy in flight, frees its tensor memory and returns, and the call
 * returns an error ("did not complete in time" / "timed out").  limit_ns = 0 restores the
 * normal waits. */
TANGERINE_API tg_status tg_debug_wait_test(int which, uint64_t limit_ns);
/* Output capacity for the next run (default: an estimate from the lattices); a run that
 * finds more vertices or faces grows the buffers and runs again (tg_batch_info.reruns). */
TANGERINE_API tg_status tg_batch_reserve(tg_batch* batch, uint64_t vertices, uint64_t faces);
TANGERINE_API tg_status tg_batch_get_info(const tg_batch* batch, tg_batch_info* out);
/* Model `model`'s mesh from the last run, copied to host memory (release with tg_mesh_free),
 * or left on the device (valid until the next run or tg_batch_free). */
TANGERINE_API tg_status tg_batch_mesh(tg_batch* batch, int model, tg_mesh* out, void* stream);
TANGERINE_API tg_status tg_batch_mesh_device(tg_batch* batch, int model, tg_device_mesh* out);

/* ---- learned distance bound ---------------------------------------------------------
 * No counterpart in the reference.  A per-tree network -- a 16-level hash grid (2 features
 * per level) feeding 3 hidden ReLU layers of 64, BF16 weights on the tensor cores with FP32
 * accumulation -- trained on the GPU by this library's own forward, backward and Adam
 * kernels on distances of the whole tree (SDFNode::Eval).  It bounds the distance for
 * brick culling: a brick is skipped only when |net(centre)| exceeds the brick's ball radius
 * plus a margin (safety x the largest error seen on held-out samples), and every kept
 * brick is evaluated exactly, so the exact program decides every sign.  Trees with a
 * non-1-Lipschitz brush (ellipsoid) are never culled by it. */
typedef struct tg_surrogate tg_surrogate;

typedef struct tg_surrogate_options
{
	int log2_table;             /* entries per level = 2^log2_table (default 18) */
	int base_resolution;        /* cells per axis, coarsest level (16) */
	int max_resolution;         /* finest level (1024) */
	float domain_min[3];        /* box the grid covers ([-2, 2]^3) */
	float domain_max[3];
	float clamp;                /* the network approximates clamp(d, -clamp, clamp) (0.5) */
	int64_t samples;            /* training samples, half uniform, half |d| < band (2^22) */
	float band;                 /* (0.05) */
	int64_t batch;              /* samples per Adam step (2^18) */
	int steps;                  /* Adam steps (1000) */
	float learning_rate;        /* (1e-2, decaying to 1e-3 over the second half) */
	int64_t validation;         /* held-out samples, same mix (2^20) */
	float safety;               /* margin = safety x max held-out error (2) */
	uint64_t seed;
} tg_surrogate_options;

typedef struct tg_surrogate_info
{
	float max_error, p99_error, mean_error;   /* held-out |net - clamp(d)| */
	float margin;                             /* safety x max_error (tg_surrogate_margin gives the one used) */
	float final_loss;                         /* mean squared error of the last batch */
	double data_seconds, train_seconds;
	int64_t samples;
	int steps;
	int resolutions[16];
	uint32_t table_size;
	uint32_t dense_levels;                    /* bit l: level l indexed densely */
	int64_t table_floats;                     /* 16 x table_size x 2 */
	int64_t mlp_floats;                       /* 10497: W1[64][32] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4 */
} tg_surrogate_info;

TANGERINE_API void tg_surrogate_default_options(tg_surrogate_options* out);
/* Allocates the network on the current device with seeded initial parameters. */
TANGERINE_API tg_status tg_surrogate_create(const tg_surrogate_options* options, tg_surrogate** out);
TANGERINE_API void tg_surrogate_free(tg_surrogate* s);
/* Builds the training set from the program's whole tree, trains, measures the held-out
 * error and sets the margin. */
TANGERINE_API tg_status tg_surrogate_fit(tg_surrogate* s, tg_program* program, void* stream);
TANGERINE_API tg_status tg_surrogate_get_info(const tg_surrogate* s, tg_surrogate_info* out);
/* Parameters as FP32 host arrays (table: level-major, entry-major, 2 features). */
TANGERINE_API tg_status tg_surrogate_get_params(tg_surrogate* s, float* table, float* mlp);
TANGERINE_API tg_status tg_surrogate_set_params(tg_surrogate* s, const float* table, const float* mlp);
/* Checkpoint and resume: the parameters with both Adam moments and the step count, the
 * info and the held-out error record behind the margins.  tg_surrogate_save with out ==
 * NULL returns the checkpoint's size in bytes; with a buffer of at least that capacity it
 * writes the checkpoint and returns its size; -1 on error.  tg_surrogate_load restores one
 * into a surrogate created with the same grid options (table size, resolutions, domain,
 * clamp; TG_ERR_INVALID otherwise or for a damaged checkpoint): tg_surrogate_train then
 * continues the same Adam schedule, and the margins are the saved ones. */
TANGERINE_API int64_t tg_surrogate_save(tg_surrogate* s, void* out, int64_t capacity);
TANGERINE_API tg_status tg_surrogate_load(tg_surrogate* s, const void* data, int64_t size);
/* Network output at n points (3 floats each); host arrays, or device when io_is_device. */
TANGERINE_API tg_status tg_surrogate_eval(tg_surrogate* s, const float* points, int64_t n, float* out, int io_is_device,
                                          void* stream);
/* Gradients of the mean squared error against clamp(d) over n samples (x, y, z, d; host
 * arrays), into host arrays shaped like the parameters; *loss = sum of squared errors. */
TANGERINE_API tg_status tg_surrogate_gradients(tg_surrogate* s, const float* samples, int64_t n, float* table_grad,
                                               float* mlp_grad, float* loss);
/* `steps` Adam steps over consecutive batches of the given samples (host x, y, z, d). */
TANGERINE_API tg_status tg_surrogate_train(tg_surrogate* s, const float* samples, int64_t n, int steps, void* stream);
/* Margin of the brick test |net(centre)| > r + margin for bricks whose ball has radius r.
 * The test is wrong only for a centre with |d| <= r where the network says more than
 * r + margin, so it comes from the held-out samples with |clamp(d)| <= r:
 * safety x max(their largest |net| - r, the held-out p99 error). */
TANGERINE_API tg_status tg_surrogate_margin(const tg_surrogate* s, float radius, float* margin);
/* Fixes the margin of the culled export for every brick size (negative: back to the
 * held-out calibration above). */
TANGERINE_API tg_status tg_surrogate_set_margin(tg_surrogate* s, float margin);
/* tg_export_mesh / tg_export_mesh_device with the network deciding which bricks to skip:
 * a brick it does not rule out also takes the exact brick test (the network saves that
 * test's cost on the bricks it rules out), unless TG_MESH_SURROGATE_ONLY is set. */
enum
{
	TG_MESH_SURROGATE_ONLY = 1u << 20,
	/* Brick evaluation: a brick inside one octree cell copies that cell's distance program
	   into shared memory (one bulk copy) and reads its records there (same results). */
	TG_MESH_STAGED = 1u << 21,
};
TANGERINE_API tg_status tg_export_mesh_surrogate(tg_program* program, tg_surrogate* s, const tg_grid* grid, uint32_t flags,
                                                 tg_mesh* out, void* stream);
TANGERINE_API tg_status tg_export_mesh_surrogate_device(tg_program* program, tg_surrogate* s, const tg_grid* grid,
                                                        uint32_t flags, tg_device_mesh* out, void* stream);

/* The batch's surrogate form: model m's bricks are culled by nets[m] (a fitted
 * tg_surrogate; NULL keeps the exact test for that model) before the launch, inside the same
 * CUDA graph; the bricks a network keeps then take the exact test too, unless flags has
 * TG_MESH_SURROGATE_ONLY.  Either way each model's mesh is the exact export's (the networks'
 * margins are conservative).  The networks must outlive the batch's runs. */
TANGERINE_API tg_status tg_batch_set_surrogates(tg_batch* batch, tg_surrogate* const* nets, int count, uint32_t flags);
/* tg_render with network steps: each ray steps by the larger of the root cube's distance
 * and the network's value less its margin (safety x the largest held-out error) until that
 * bound falls to the margin, then by SDFNode::RayMarch's exact whole-tree steps; hits are
 * the exact program's and are shaded with the whole tree's gradient and material.  The
 * step budget (max_steps) covers both kinds of step. */
TANGERINE_API tg_status tg_render_surrogate(tg_program* program, tg_surrogate* s, const tg_camera* cameras, int count, int width,
                                            int height, int max_steps, float epsilon, float* depth, float* normals,
                                            uint8_t* colors, int out_is_device, void* stream);
/* Network iterations (per ray, summed) and exact steps of the last tg_render_surrogate. */
TANGERINE_API tg_status tg_last_render_steps(uint64_t* network_steps, uint64_t* exact_steps);
/* Check of the tensor-core operand layouts: D = A B^T through the descriptors the network
 * kernels use (mode 0: a 128x64, b 64x64, both K-major, D 128x64; mode 1: D = a^T b for
 * a 128x128, b 128x144, D 128x144; mode 2: D = a b for a 128x64, b 64x64, D 128x64).
 * Host FP32 arrays, inputs rounded to BF16. */
TANGERINE_API tg_status tg_debug_mma(int mode, const float* a, const float* b, float* d);

/* Check of the GPU's float evaluation of the smooth-blend term against the reference's
 * double expression on n seeded inputs (x2 signs): counts[0] compared, counts[1] differing
 * (must be 0), counts[2] sent to the double path. */
TANGERINE_API tg_status tg_debug_blend_check(uint64_t n, uint64_t seed, uint64_t* counts);
/* Check of the paired FP32 arithmetic the distance interpreters use (FADD2 / FMUL2, two
 * points per instruction) against the scalar formulas on n seeded inputs: counts[0] inputs,
 * counts[1..9] lanes differing in bits (all must be 0) for: one add, one multiply, a product
 * then a sum, sphere, box, torus, cylinder, plane, the affine transform. */
TANGERINE_API tg_status tg_debug_pair_check(uint64_t n, uint64_t seed, uint64_t* counts);

TANGERINE_API const char* tg_last_error(void);
TANGERINE_API const char* tg_version(void);

#ifdef __cplusplus
}
#endif

#endif
