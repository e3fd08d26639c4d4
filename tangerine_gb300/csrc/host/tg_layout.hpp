// Device-visible layout of a compiled tree, shared by the host compiler and the kernels.
//
// A compiled tree ("program") lives in one device allocation:
//   OctNode  nodes[node_count]      the export octree, depth-first, root first
//   float4   code[code_quads]       every node's two programs, 16-byte records
//   uchar4   colors[material_count] resolved material colour bytes
//   float4   material_rgb[material_count]  each material's stored RGB (alpha 1)
//
// Each octree node carries two programs for its clipped subtree:
//  * the distance program: Tangerine's postfix program (SDFNode::Compile), with each
//    brush's [Matrix|Offset] brush [ScaleField] words fused into one record of 1..6 quads;
//  * the surface program: the same subtree in the form SDFNode::Eval walks it (quaternion
//    inverse transforms, per-brush materials) for gradient normals and colours.
#pragma once

#include <cstdint>

namespace tg
{
	// Record flags (bits 8.. of a record's first word; bits 0..7 hold the opcode).
	enum : uint32_t
	{
		RecMatrix = 1u << 8,        // distance brush: 3 quads of inverse-matrix rows follow
		RecOffset = 1u << 9,        // distance brush: 1 quad (-translation) follows
		RecScale = 1u << 10,        // distance brush: 1 quad (scale) follows
		RecLhsPaint = 1u << 11,     // surface set op: left operand has paint
		RecRhsPaint = 1u << 12,     // surface set op: right operand has paint
		RecNegative = 1u << 13,     // surface stencil: override applies inside the mask
		RecThenSet = 1u << 14,      // distance brush: the next record is the set operator whose
		                            // right operand this brush is (applied in the same step)
	};

	// Extra opcodes used only by surface programs.
	enum : uint32_t
	{
		OpMaskBegin = 32,           // quad: {op, skip quads (distance-only evaluation jumps)}
		OpStencilEnd = 33,          // quad: {op|flags, material index}
	};

	constexpr int kMaxStack = 32;   // deepest postfix stack a program may need
	constexpr int32_t kNodeTerminus = 1;
	// The cell has no evaluator: SDFOctree::Populate found all eight children empty after
	// the cell itself was kept (meshing octree's second stage only).  Its programs are a
	// lone stop record.
	constexpr int32_t kNodeNoEvaluator = 2;

	struct OctNode
	{
		float Pivot[3];
		int32_t Flags;              // bit 0: terminus; bit 1: no evaluator; bits 8..15: octants
		                            // whose clip returned null (the evaluator exceeds the
		                            // octant sphere's radius)
		int32_t Child[8];           // -1: no child there
		int32_t DistanceCode;       // quad offset of the distance program
		int32_t SurfaceCode;        // quad offset of the surface program
		int32_t StackSize;
		float ClipRadius;           // radius of the sphere the cell's evaluator was clipped to;
		                            // negated when the program is not 1-Lipschitz (ellipsoid)
	};
	static_assert(sizeof(OctNode) == 64, "OctNode is one 64-byte line");

	// Export lattice: point (i, j, k) sits at (X0 + i*DX, Y0 + j*DY, Z0 + k*DZ).
	struct GridSpec
	{
		float X0, Y0, Z0;
		float DX, DY, DZ;       // step per axis
		int NX, NY, NZ;         // lattice points per axis; cells are one fewer
	};

	struct ProgramHeader
	{
		int32_t NodeCount;
		int32_t CodeQuads;
		int32_t MaterialCount;
		int32_t HasPaint;           // root evaluator HasPaint(): colours are exported
		int32_t MaxStack;
		int32_t FullSurfaceCode;    // quad offset of the whole tree's surface program
		int32_t Lipschitz;          // 1 when every brush is 1-Lipschitz (no ellipsoid)
		int32_t Reserved;
	};
}
