// Export octree and program compilation (host side).
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "tg_layout.hpp"
#include "tg_tree.hpp"

namespace tg
{
	// SDFOctree (sdf_evaluator.cpp:1609-1783) with the export settings: target size 0.25,
	// coalescing on, no depth limit.
	struct Octree
	{
		struct Cell
		{
			AABB Bounds;
			Vec3 Pivot;
			float ClipRadius = 0.0f;
			uint32_t NullOctants = 0;   // children whose clip returned null
			bool Terminus = false;
			bool Incomplete = false;
			int EvaluatorLeaves = 0;
			NodeRef Evaluator;
			int Children[8] = { -1, -1, -1, -1, -1, -1, -1, -1 };
		};
		std::vector<Cell> Cells;   // depth-first, root first

		// The root cell as soon as its clip is done, before the levels below it are built:
		// its pivot, clip radius and evaluator are already the ones Cells[0] ends with.
		using RootSeen = std::function<void(const Vec3& pivot, float clip_radius, const NodeRef& evaluator)>;
		// Returns false (and leaves Cells empty) when the tree has infinite or empty
		// bounds, or clips away entirely, as SDFOctree::Create returns nullptr.
		bool Build(const NodeRef& root, float target_size = 0.25f, bool coalesce = true, int max_depth = -1,
			const RootSeen* on_root = nullptr);
		// Sodapop's meshing octree (sodapop.cpp:565-567): SDFOctree::Create(.25, false, 3),
		// then every cell left incomplete at depth 3 populated on its own with
		// Populate(false, 3, -1).  The second stage does not revisit the ancestors, so they
		// keep the bounds they took at depth 3, and a populated cell whose eight children
		// all clip away stays in place without an evaluator.
		bool BuildMeshing(const NodeRef& root);
		int Descend(Vec3 p) const;                 // Descend(Point, Exact=true)
	};

	// Distance program words exactly as Tangerine's SDFInterpreter holds them
	// (SDFNode::Compile + Stop), for checking against the reference.
	std::vector<uint32_t> CompileReferenceWords(const Node& tree);
	bool HasNonLipschitzBrush(const Node& tree);

	struct DeferredSurfaces;   // what a compile needs to emit the surface programs later

	struct CompiledTree
	{
		ProgramHeader Header{};
		std::vector<OctNode> Nodes;
		// The record quads (4 floats each) in the pieces the emitters wrote them in; laid
		// end to end they are the program image (CopyCode).
		std::vector<std::vector<float>> CodeChunks;
		size_t CodeFloats = 0;
		void CopyCode(float* dst) const;
		// Set while the surface programs are still to be emitted (a compile that deferred
		// them): their places in the image are laid out and zero-filled, every offset,
		// stack size and the distance programs are final (FinishSurfaces).
		std::shared_ptr<DeferredSurfaces> Pending;
		std::vector<uint8_t> Colors;      // 4 bytes per material
		std::vector<float> MaterialRgb;   // 4 floats per material: stored RGB, 1
		AABB Bounds{};                    // root evaluator bounds
		AABB OctreeBounds{};              // the octree root cell's bounds
		std::vector<AABB> LeafBounds;     // terminus cells with an evaluator (meshing octree)
		double BuildSeconds = 0.0;
		double OctreeSeconds = 0.0;       // of which the octree (clips, merges)
		int64_t DistanceQuadsTotal = 0;
	};

	// The export octree's root cell on its own, as a one-cell program image: Node is the
	// compiled tree's node 0 (terminus, no children, its distance program at quad 0,
	// StackSize that program's depth) and Code that distance program with its stop
	// record -- the same records the compiled tree gives node 0.  It exists a few tens of
	// microseconds into the compile, long before the octree below it: the root's program
	// has the whole tree's sign everywhere in the root sphere, so the exact brick test can
	// run on it while the host builds the rest.
	struct RootProgram
	{
		OctNode Node{};
		std::vector<float> Code;
	};
	using RootHook = std::function<void(const RootProgram&)>;

	enum class OctreeKind { Export, Meshing };
	// Builds the octree of the given kind (Export: target 0.25 with coalescing, as the
	// export and the point queries use; Meshing: Octree::BuildMeshing) and compiles every
	// cell's clipped subtree.  `on_root` (Export only) is called on the compiling thread
	// with the root cell's program as soon as the root is clipped.  `defer_surfaces`: the
	// surface programs (read only by the per-vertex normal and colour pass and by queries
	// of the surface) are laid out but left for FinishSurfaces.
	bool CompileTree(const NodeRef& root, CompiledTree& out, std::string& error, OctreeKind kind = OctreeKind::Export,
		const RootHook* on_root = nullptr, bool defer_surfaces = false);
	// Emits the surface programs a deferred compile left out, on the worker pool, into
	// `image` (the whole code image as CopyCode lays it out: quad 0 first) or, with
	// image == nullptr, into CodeChunks.  Only the surface programs' places are written.
	// No-op when nothing is pending; false (with `error`) if a program's size is not the
	// one laid out.
	bool FinishSurfaces(CompiledTree& t, float* image, std::string& error);
}
