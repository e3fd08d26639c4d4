// CSG trees: the host-side model of Tangerine's SDFNode hierarchy
// (tangerine/sdf_evaluator.h:171-264).  A tree is built from brushes and operators,
// mutated by Move/Rotate/Scale/ApplyMaterial while it is being assembled, and then only
// read: clipping makes new nodes that share the unchanged subtrees.
#pragma once

#include <atomic>
#include <cstdint>
#include <memory>
#include <vector>

#include "tg_math.hpp"
#include "tg_sdfmath.hpp"

namespace tg
{
	// A material is an sRGB base colour; two materials are the same material only if they
	// are the same object (MaterialInterface::operator==, sdf_evaluator.h:66-67).
	struct Material
	{
		float Rgb[3];
	};
	using MaterialRef = std::shared_ptr<const Material>;

	enum class NodeKind : uint8_t { Brush, Set, Flate, Stencil };

	struct Node;

	// Intrusive reference: the C ABI hands these out as plain pointers.  A reference may
	// also be borrowed (tagged in the pointer's low bit): it counts nothing and keeps
	// nothing alive.  The octree's clipped trees borrow the nodes of the tree they were
	// clipped from, which outlives them, so that threads clipping in parallel do not all
	// write the shared nodes' counters.
	class NodeRef
	{
	public:
		NodeRef() = default;
		explicit NodeRef(Node* adopt) : P(reinterpret_cast<uintptr_t>(adopt)) {}
		NodeRef(const NodeRef& o);
		NodeRef(NodeRef&& o) noexcept : P(o.P) { o.P = 0; }
		NodeRef& operator=(NodeRef o) { std::swap(P, o.P); return *this; }
		~NodeRef();
		Node* get() const { return reinterpret_cast<Node*>(P & ~kBorrowed); }
		Node* operator->() const { return get(); }
		Node& operator*() const { return *get(); }
		explicit operator bool() const { return P != 0; }
		bool Borrowed() const { return (P & kBorrowed) != 0; }
		// A counted pointer for the caller (a borrowed reference takes a count first).
		Node* release();
		static NodeRef Share(Node* n);
		static NodeRef Borrow(const Node* n);
	private:
		static constexpr uintptr_t kBorrowed = 1;
		uintptr_t P = 0;
	};

	struct Node
	{
		std::atomic<int> Refs{ 1 };
		uint32_t ClipMark = 0;   // the clip call that made this node (0: not made by a clip)
		NodeKind Kind = NodeKind::Brush;
		uint32_t Op = OpStop;
		int StackSize = 1;

		// Brush
		float Params[3] = { 0.0f, 0.0f, 0.0f };
		float Args[3] = { 0.0f, 0.0f, 0.0f };   // the constructor's arguments (tree specs replay them)
		AABB BrushBox{};
		Transform Xf;
		MaterialRef Mat;

		// Set (Lhs, Rhs, Threshold), Flate (Lhs = child, Threshold = radius),
		// Stencil (Lhs = child, Mask, Mat, Negative).
		NodeRef Lhs, Rhs, Mask;
		float Threshold = 0.0f;
		bool Negative = false;

		float Eval(Vec3 p) const;
		// `borrow`: the result borrows the nodes it keeps from this tree (only the nodes the
		// clip rebuilt are counted), so it must not outlive this tree.
		NodeRef Clip(Vec3 p, float radius, bool borrow = false) const;
		// Clip to eight spheres at once (the same result as eight Clip calls).
		void Clip8(const Vec3 (&p)[8], const float (&radius)[8], NodeRef (&out)[8], bool borrow = false) const;
		AABB Bounds() const;
		AABB InnerBounds() const;
		void Move(Vec3 by);
		void Rotate(Quat by);
		void Scale(float by);
		void ApplyMaterial(const MaterialRef& m, bool force);
		bool HasPaint() const;
		bool HasFiniteBounds() const;
		int LeafCount() const;
		bool Equals(const Node& o) const;
		Vec3 Gradient(Vec3 p) const;
		const Material* GetMaterial(Vec3 p) const;   // nullptr: the default white
	private:
		AABB BoundsImpl(bool inner) const;
	};

	struct RayHit
	{
		bool Hit;
		float Travel;
		Vec3 Position;
	};
	RayHit RayMarch(const Node& tree, Vec3 start, Vec3 dir, int max_iterations, float epsilon);

	// Constructors and helpers with the SDF:: semantics (sdf_evaluator.cpp:1169-1372).
	namespace SDF
	{
		NodeRef Sphere(float radius);
		NodeRef Ellipsoid(float rx, float ry, float rz);
		NodeRef Box(float ex, float ey, float ez);
		NodeRef Torus(float major, float minor);
		NodeRef Cylinder(float radius, float extent);
		NodeRef Plane(float nx, float ny, float nz);
		NodeRef Cone(float radius, float height);
		NodeRef Coninder(float radius_low, float radius_high, float height);
		NodeRef Union(NodeRef lhs, NodeRef rhs);
		NodeRef Diff(NodeRef lhs, NodeRef rhs);
		NodeRef Inter(NodeRef lhs, NodeRef rhs);
		NodeRef BlendUnion(float k, NodeRef lhs, NodeRef rhs);
		NodeRef BlendDiff(float k, NodeRef lhs, NodeRef rhs);
		NodeRef BlendInter(float k, NodeRef lhs, NodeRef rhs);
		NodeRef Flate(NodeRef node, float radius);
		NodeRef Stencil(NodeRef node, NodeRef mask, MaterialRef material, bool apply_to_negative);
		void Align(Node& tree, Vec3 anchors);
		void RotateX(Node& tree, float degrees);
		void RotateY(Node& tree, float degrees);
		void RotateZ(Node& tree, float degrees);
		NodeRef MakeSet(uint32_t op, NodeRef lhs, NodeRef rhs, float k);
	}

	// Builds a tree from a postfix tree spec (the word stream tangerine_gb300.workloads
	// writes).  Returns an empty ref and fills `error` on a malformed spec.
	NodeRef BuildFromSpec(const float* spec, int count, const char** error);
	// The spec that rebuilds this tree exactly: each brush with its whole transform (the
	// transform op) and material, set operators in their stored operand order (already
	// left-leaning, so the replay keeps it), flates and stencils.
	void WriteSpec(const Node& tree, std::vector<float>& out);
	// SDFNode::Copy (sdf_evaluator.cpp:480-483, 617-620, 852-855, 1077-1080): a new tree of
	// new nodes with the same parameters, transforms and materials.
	NodeRef CopyTree(const Node& tree);
}
