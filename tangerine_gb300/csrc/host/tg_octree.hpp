// Export octree and program compilation (host side).
#pragma once

#include <cstdint>
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

		// Returns false (and leaves Cells empty) when the tree has infinite or empty
		// bounds, or clips away entirely, as SDFOctree::Create returns nullptr.
		bool Build(const NodeRef& root, float target_size = 0.25f, bool coalesce = true, int max_depth = -1);
		int Descend(Vec3 p) const;                 // Descend(Point, Exact=true)
	};

	// Distance program words exactly as Tangerine's SDFInterpreter holds them
	// (SDFNode::Compile + Stop), for checking against the reference.
	std::vector<uint32_t> CompileReferenceWords(const Node& tree);
	bool HasNonLipschitzBrush(const Node& tree);

	struct CompiledTree
	{
		ProgramHeader Header{};
		std::vector<OctNode> Nodes;
		std::vector<float> Code;          // 4 floats per quad
		std::vector<uint8_t> Colors;      // 4 bytes per material
		AABB Bounds{};                    // root evaluator bounds
		double BuildSeconds = 0.0;
		int64_t DistanceQuadsTotal = 0;
	};

	bool CompileTree(const NodeRef& root, CompiledTree& out, std::string& error);
}
