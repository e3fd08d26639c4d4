/*
 * Test infrastructure only -- the CPU oracle for the GPU export path.
 *
 * A plain-C restatement of Tangerine's CPU path from a CSG tree to an exported mesh:
 * SDFNode Eval/Clip/Bounds/Compile (tangerine/sdf_evaluator.cpp:165-1372), the postfix
 * interpreter (sdf_evaluator.cpp:1386-1605), SDFOctree (sdf_evaluator.cpp:1609-2005),
 * naive surface nets (third_party/naive-surface-nets/src/surface_nets.cpp:829-1122),
 * gradient normals and material colours (tangerine/export.cpp:283-317) and RayMarch
 * (sdf_evaluator.cpp:336-353).  Every float operation follows the reference's (and glm
 * 0.9.9.8's) operation order, and the library is built with -ffp-contract=off, so on the
 * golden fixtures written by the reference itself it is bit-exact.
 *
 * Only tests/, the smoke check and bench.py's CPU-baseline leg may load this library.
 * The product never links it.
 */
#ifndef TG_ORACLE_H
#define TG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tgo_tree tgo_tree;
typedef struct tgo_octree tgo_octree;

/* Tree spec: postfix float32 word stream (opcodes are small integers stored as floats).
 * The op codes are listed in tg_oracle.c (SPEC_*).  Returns NULL on a malformed spec. */
tgo_tree* tgo_build(const float* spec, int count);
void tgo_free(tgo_tree* tree);
void tgo_free_buffer(void* buffer);

int tgo_stack_size(tgo_tree* tree);
int tgo_has_paint(tgo_tree* tree);
int tgo_has_finite_bounds(tgo_tree* tree);
int tgo_leaf_count(tgo_tree* tree);
void tgo_bounds(tgo_tree* tree, float* out6, int inner);

void tgo_eval(tgo_tree* tree, int64_t n, const float* points, float* out);
void tgo_gradient(tgo_tree* tree, int64_t n, const float* points, float* out);
void tgo_color(tgo_tree* tree, int64_t n, const float* points, uint8_t* out);
int tgo_compile(tgo_tree* tree, uint32_t* out, int capacity);
void tgo_interp_eval(tgo_tree* tree, int64_t n, const float* points, float* out);
tgo_tree* tgo_clip(tgo_tree* tree, float x, float y, float z, float radius);
int tgo_equal(tgo_tree* a, tgo_tree* b);

tgo_octree* tgo_octree_create(tgo_tree* tree, float target_size, int coalesce, int max_depth);
/* Sodapop's meshing octree: create(.25, no coalescing, depth 3), then each incomplete
 * cell populated without a depth limit (sodapop.cpp:565-569). */
tgo_octree* tgo_meshing_octree_create(tgo_tree* tree);
void tgo_octree_free(tgo_octree* octree);
int tgo_octree_dump(tgo_octree* octree, float** nodes, int32_t** children, uint32_t** words, int* word_count);
void tgo_octree_eval(tgo_octree* octree, int64_t n, const float* points, int exact, float* out);
void tgo_octree_gradient(tgo_octree* octree, int64_t n, const float* points, float* out);
void tgo_octree_color(tgo_octree* octree, int64_t n, const float* points, uint8_t* out);
int tgo_octree_has_paint(tgo_octree* octree);
void tgo_octree_grid(tgo_octree* octree, float x0, float y0, float z0, float dx, float dy, float dz,
                     int64_t nx, int64_t ny, int64_t nz, int threads, float* out);

/* Naive surface nets over the octree's exact distances on the grid
 * (x0 + i*dx, ...), sx*sy*sz cells.  Vertices are numbered in (k, j, i) cell order, which
 * is the order the reference's serial pstl backend produces.  faithful=1 evaluates 8
 * corners per cell and 4 per face like the reference; faithful=0 evaluates each lattice
 * corner once.  Buffers are malloc'd (tgo_free_buffer).  Returns the vertex count, or -1
 * on an unsupported (non-cubic) grid. */
int64_t tgo_surface_nets(tgo_octree* octree, float x0, float y0, float z0, float dx, float dy, float dz,
                         int64_t sx, int64_t sy, int64_t sz, int threads, int faithful,
                         float** vertices, uint64_t** cubes, uint64_t** faces, int64_t* face_count,
                         double* seconds);

/* Per-vertex gradient normals and colour bytes as WritePLY(Octree, ...) computes them. */
void tgo_vertex_attributes(tgo_octree* octree, int64_t n, const float* vertices, int threads,
                           float* normals, uint8_t* colors);

void tgo_raymarch(tgo_tree* tree, int64_t n, const float* origins, const float* dirs,
                  int max_iterations, float epsilon, int threads,
                  uint8_t* hit, float* travel, float* position);

/* Lua's magnet cast (mode 1) and SDFModel::RayMarch in a model frame (mode 2: frame = quat
 * w x y z, translation xyz, scale), serially. */
void tgo_ray_query(tgo_tree* tree, int mode, const float* frame, int64_t n, const float* origins, const float* dirs,
                   int iterations, float epsilon, uint8_t* hit, float* travel, float* position);
int tgo_hardware_threads(void);
/* Sodapop's meshing chain (sodapop.cpp:562-897) over the tree, serially: returns the vertex
 * count (-1 without an octree); positions/normals (3 floats), colours (4 floats), faces (3
 * indices) are malloc'd (release with tgo_free_buffer); grid_out gets x y z dx dy dz sx sy sz. */
int64_t tgo_sodapop(tgo_tree* tree, float density, float** positions, float** normals, float** colors, uint64_t** faces,
	int64_t* face_count, float* grid_out);

/* PointCloudExportThread (export.cpp:384-480) in cell order: cell centres of the
 * ceil((max - min) / step) lattice with |octree distance| < |step / 2|, refined by
 * `refine` gradient steps and kept within their voxel.  points: 3 floats per point, cells:
 * the lattice cell number (malloc'd).  Returns the point count. */
int64_t tgo_point_cloud(tgo_octree* octree, const float* min3, const float* max3, const float* step3, int refine,
                        float** points, int32_t** cells);
/* VoxExport's voxel test (magica.cpp:27-69) in cell order: voxels gets x, y, z, colour index
 * per voxel (malloc'd); size_out the lattice, radius_out the half-voxel radius. */
int64_t tgo_vox(tgo_tree* tree, float grid_size, int color_index, int32_t* size_out, float* radius_out, int32_t** voxels);

#ifdef __cplusplus
}
#endif

#endif
