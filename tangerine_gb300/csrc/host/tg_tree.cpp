// CSG tree semantics (see tg_tree.hpp).  Each member names the reference behaviour it
// reproduces; the float arithmetic matches the reference operation for operation.
#include "tg_tree.hpp"

#include <cmath>
#include <limits>
#include <unordered_map>
#include <vector>

namespace tg
{
	NodeRef::NodeRef(const NodeRef& o) : P(o.P)
	{
		if (P && !Borrowed()) get()->Refs.fetch_add(1, std::memory_order_relaxed);
	}

	NodeRef::~NodeRef()
	{
		if (P && !Borrowed() && get()->Refs.fetch_sub(1, std::memory_order_acq_rel) == 1) delete get();
	}

	Node* NodeRef::release()
	{
		Node* r = get();
		if (Borrowed() && r) r->Refs.fetch_add(1, std::memory_order_relaxed);
		P = 0;
		return r;
	}

	NodeRef NodeRef::Share(Node* n)
	{
		if (n) n->Refs.fetch_add(1, std::memory_order_relaxed);
		return NodeRef(n);
	}

	NodeRef NodeRef::Borrow(const Node* n)
	{
		NodeRef r;
		if (n) r.P = reinterpret_cast<uintptr_t>(n) | kBorrowed;
		return r;
	}

	// Virtual Eval (sdf_evaluator.cpp:463-466, 598-601, 774-780, 1059-1062): brushes map
	// the point through the inverse transform (quaternion form) and rescale the distance.
	float Node::Eval(Vec3 p) const
	{
		switch (Kind)
		{
		case NodeKind::Brush: return BrushDistance(Op, Params, Xf.ApplyInv(p)) * Xf.Scalation;
		case NodeKind::Set: return SetDistance(Op, Lhs->Eval(p), Rhs->Eval(p), Threshold);
		case NodeKind::Flate: return Lhs->Eval(p) - Threshold;
		case NodeKind::Stencil: return Lhs->Eval(p);
		}
		return 0.0f;
	}

	namespace
	{
		// Distances of every subtree at one point, each computed once.  The reference's
		// Clip calls the virtual Eval at every level of the recursion, re-evaluating each
		// subtree once per ancestor; caching gives the same floats (same operations, same
		// order) in time linear in the tree.
		struct PointEvaluations
		{
			// Open-addressing table keyed by node address; entries of earlier points are
			// told apart by a per-thread epoch, so no clearing between clips.
			struct Slot
			{
				const Node* Key;
				float Value;
				uint32_t Epoch;
			};
			static thread_local std::vector<Slot> Table;
			static thread_local uint32_t Epoch;
			Vec3 P;
			uint32_t Used = 0;

			explicit PointEvaluations(Vec3 p) : P(p)
			{
				if (Table.empty()) Table.assign(4096, Slot{ nullptr, 0.0f, 0 });
				if (++Epoch == 0)
				{
					for (Slot& s : Table) s.Epoch = 0;
					Epoch = 1;
				}
			}

			static size_t HashOf(const Node* n, size_t mask)
			{
				uint64_t x = (uint64_t)(uintptr_t)n;
				x ^= x >> 33;
				x *= 0xff51afd7ed558ccdull;
				x ^= x >> 33;
				return (size_t)x & mask;
			}

			bool Find(const Node* n, float& v) const
			{
				const size_t mask = Table.size() - 1;
				for (size_t i = HashOf(n, mask);; i = (i + 1) & mask)
				{
					const Slot& s = Table[i];
					if (s.Epoch != Epoch) return false;
					if (s.Key == n) { v = s.Value; return true; }
				}
			}

			void Insert(const Node* n, float v)
			{
				if (2 * (Used + 1) > Table.size()) Grow();
				const size_t mask = Table.size() - 1;
				size_t i = HashOf(n, mask);
				while (Table[i].Epoch == Epoch) i = (i + 1) & mask;
				Table[i] = Slot{ n, v, Epoch };
				++Used;
			}

			void Grow()
			{
				std::vector<Slot> old;
				old.swap(Table);
				Table.assign(old.size() * 2, Slot{ nullptr, 0.0f, 0 });
				const size_t mask = Table.size() - 1;
				for (const Slot& s : old)
				{
					if (s.Epoch != Epoch) continue;
					size_t i = HashOf(s.Key, mask);
					while (Table[i].Epoch == Epoch) i = (i + 1) & mask;
					Table[i] = s;
				}
			}

			float At(const Node& n)
			{
				float v = 0.0f;
				if (Find(&n, v)) return v;
				switch (n.Kind)
				{
				case NodeKind::Brush: v = BrushDistance(n.Op, n.Params, n.Xf.ApplyInv(P)) * n.Xf.Scalation; break;
				case NodeKind::Set: v = SetDistance(n.Op, At(*n.Lhs), At(*n.Rhs), n.Threshold); break;
				case NodeKind::Flate: v = At(*n.Lhs) - n.Threshold; break;
				case NodeKind::Stencil: v = At(*n.Lhs); break;
				}
				Insert(&n, v);
				return v;
			}
		};

		thread_local std::vector<PointEvaluations::Slot> PointEvaluations::Table;
		thread_local uint32_t PointEvaluations::Epoch = 0;

		// The same evaluations at eight points at once (the eight children of an octree
		// cell clip their parent's tree at their own pivots): one walk of the tree, one
		// table lookup per node, one quaternion inverse per brush for all eight points.
		struct Evaluations8
		{
			struct Slot
			{
				const Node* Key;
				uint32_t Index;
				uint32_t Epoch;
			};
			static thread_local std::vector<Slot> Table;
			static thread_local uint32_t Epoch;
			Vec3 P[8];
			std::vector<float> Values;
			uint32_t Used = 0;

			explicit Evaluations8(const Vec3 (&p)[8])
			{
				for (int i = 0; i < 8; ++i) P[i] = p[i];
				if (Table.empty()) Table.assign(4096, Slot{ nullptr, 0, 0 });
				if (++Epoch == 0)
				{
					for (Slot& s : Table) s.Epoch = 0;
					Epoch = 1;
				}
				Values.reserve(8 * 1024);
			}

			static size_t HashOf(const Node* n, size_t mask)
			{
				uint64_t x = (uint64_t)(uintptr_t)n;
				x ^= x >> 33;
				x *= 0xff51afd7ed558ccdull;
				x ^= x >> 33;
				return (size_t)x & mask;
			}

			void Grow()
			{
				std::vector<Slot> old;
				old.swap(Table);
				Table.assign(old.size() * 2, Slot{ nullptr, 0, 0 });
				const size_t mask = Table.size() - 1;
				for (const Slot& s : old)
				{
					if (s.Epoch != Epoch) continue;
					size_t i = HashOf(s.Key, mask);
					while (Table[i].Epoch == Epoch) i = (i + 1) & mask;
					Table[i] = s;
				}
			}

			// Index (into Values, x8) of the node's eight values, computed on first use.
			uint32_t Index(const Node& n)
			{
				{
					const size_t mask = Table.size() - 1;
					for (size_t i = HashOf(&n, mask);; i = (i + 1) & mask)
					{
						const Slot& s = Table[i];
						if (s.Epoch != Epoch) break;
						if (s.Key == &n) return s.Index;
					}
				}
				float v[8];
				switch (n.Kind)
				{
				case NodeKind::Brush:
				{
					// Transform::ApplyInv with the rotation's inverse taken once.
					const Quat inv = Inverse(n.Xf.Rotation);
					for (int i = 0; i < 8; ++i)
					{
						const Vec3 q = tg::Rotate(inv, P[i] - n.Xf.Translation) / n.Xf.Scalation;
						v[i] = BrushDistance(n.Op, n.Params, q) * n.Xf.Scalation;
					}
					break;
				}
				case NodeKind::Set:
				{
					const uint32_t li = Index(*n.Lhs);
					float l[8];
					for (int i = 0; i < 8; ++i) l[i] = Values[8 * li + i];
					const uint32_t ri = Index(*n.Rhs);
					for (int i = 0; i < 8; ++i) v[i] = SetDistance(n.Op, l[i], Values[8 * ri + i], n.Threshold);
					break;
				}
				case NodeKind::Flate:
				{
					const uint32_t ci = Index(*n.Lhs);
					for (int i = 0; i < 8; ++i) v[i] = Values[8 * ci + i] - n.Threshold;
					break;
				}
				case NodeKind::Stencil:
				{
					const uint32_t ci = Index(*n.Lhs);
					for (int i = 0; i < 8; ++i) v[i] = Values[8 * ci + i];
					break;
				}
				}
				const uint32_t index = (uint32_t)(Values.size() / 8);
				Values.insert(Values.end(), v, v + 8);
				if (2 * (Used + 1) > Table.size()) Grow();
				const size_t mask = Table.size() - 1;
				size_t i = HashOf(&n, mask);
				while (Table[i].Epoch == Epoch) i = (i + 1) & mask;
				Table[i] = Slot{ &n, index, Epoch };
				++Used;
				return index;
			}
		};

		thread_local std::vector<Evaluations8::Slot> Evaluations8::Table;
		thread_local uint32_t Evaluations8::Epoch = 0;

		// The clip works on plain pointers: an untouched subtree is the input node itself, and
		// only rebuilt nodes are allocated, kept alive in `keep` until the caller holds the
		// result.  Reference counts (atomics on nodes that every thread's clips share) are
		// touched only for rebuilt nodes' operands and the final result, and not at all for
		// the input tree's nodes when the result borrows them.
		std::atomic<uint32_t> gClipCalls{ 0 };

		struct ClipScratch
		{
			std::vector<NodeRef> Keep;
			bool BorrowInputs = false;
			uint32_t Mark = 0;
			explicit ClipScratch(bool borrow) : BorrowInputs(borrow)
			{
				if (borrow)
				{
					do Mark = gClipCalls.fetch_add(1, std::memory_order_relaxed) + 1;
					while (Mark == 0);
				}
			}
			const Node* Hold(NodeRef n)
			{
				n->ClipMark = Mark;
				const Node* raw = n.get();
				Keep.push_back(std::move(n));
				return raw;
			}
			// A reference to a node of the clip's result: counted for the nodes this clip
			// made (Keep lets go of them), borrowed for the input's nodes when the caller
			// asked for that.  A mark left by another clip only makes a reference counted.
			NodeRef Ref(const Node* n) const
			{
				if (BorrowInputs && n->ClipMark != Mark) return NodeRef::Borrow(n);
				return NodeRef::Share(const_cast<Node*>(n));
			}
		};

		// A set node whose clipped operands are its own operands is kept as it is (the
		// node MakeSet would build from them is the same node).
		const Node* RebuildSet(const Node& n, const Node* l, const Node* r, ClipScratch& cs)
		{
			if (l == n.Lhs.get() && r == n.Rhs.get()) return &n;
			return cs.Hold(SDF::MakeSet(n.Op, cs.Ref(l), cs.Ref(r), n.Threshold));
		}

		// Clip (sdf_evaluator.cpp:468-478, 603-615, 782-850, 1064-1075): the part of the tree
		// that can matter inside the sphere (p, radius).  Union keeps whichever side is near,
		// Diff keeps its left side, Inter needs both; blending widens the sphere by k.
		template<typename Ev>
		const Node* ClipAt(const Node& n, float radius, Ev& ev, ClipScratch& cs)
		{
			switch (n.Kind)
			{
			case NodeKind::Brush:
				return ev.At(n) <= radius ? &n : nullptr;
			case NodeKind::Stencil:
			{
				const Node* child = ClipAt(*n.Lhs, radius, ev, cs);
				if (!child) return nullptr;
				return cs.Hold(SDF::Stencil(cs.Ref(child), cs.BorrowInputs ? NodeRef::Borrow(n.Mask.get()) : n.Mask, n.Mat, n.Negative));
			}
			case NodeKind::Flate:
			{
				if (!(ev.At(n) <= radius)) return nullptr;
				const Node* child = ClipAt(*n.Lhs, radius + n.Threshold, ev, cs);
				if (!child) return nullptr;
				return cs.Hold(SDF::Flate(cs.Ref(child), n.Threshold));
			}
			case NodeKind::Set:
			{
				if (!(ev.At(n) <= radius)) return nullptr;
				const bool unionFamily = (n.Op == OpUnion || n.Op == OpBlendUnion);
				const bool diffFamily = (n.Op == OpDiff || n.Op == OpBlendDiff);
				if (IsBlendOp(n.Op))
				{
					const float wide = radius + n.Threshold;
					const Node* l = ClipAt(*n.Lhs, wide, ev, cs);
					const Node* r = ClipAt(*n.Rhs, wide, ev, cs);
					if (l && r) return RebuildSet(n, l, r, cs);
					if (!unionFamily && !diffFamily) return nullptr;
				}
				const Node* l = ClipAt(*n.Lhs, radius, ev, cs);
				const Node* r = ClipAt(*n.Rhs, radius, ev, cs);
				if (l && r) return RebuildSet(n, l, r, cs);
				if (unionFamily) return l ? l : r;
				if (diffFamily) return l;
				return nullptr;
			}
			}
			return nullptr;
		}

		// ClipAt for the eight spheres of an Evaluations8 at once: out[i] for each lane i set
		// in `lanes` (the other entries are left alone).  Every lane takes the branches and
		// rebuilds the nodes its own ClipAt would, in the same order of operands; the tree is
		// walked once for all of them, and each node's eight values are looked up once per
		// visit instead of once per lane.
		void ClipAt8(const Node& n, const float (&radius)[8], uint32_t lanes, const Node* (&out)[8], Evaluations8& ev,
			ClipScratch& cs)
		{
			float v[8];
			if (n.Kind != NodeKind::Stencil)
			{
				const uint32_t at = ev.Index(n);
				for (int i = 0; i < 8; ++i) v[i] = ev.Values[8 * (size_t)at + (size_t)i];
			}
			switch (n.Kind)
			{
			case NodeKind::Brush:
				for (int i = 0; i < 8; ++i)
					if ((lanes >> i) & 1u) out[i] = v[i] <= radius[i] ? &n : nullptr;
				return;
			case NodeKind::Stencil:
			{
				const Node* child[8];
				ClipAt8(*n.Lhs, radius, lanes, child, ev, cs);
				for (int i = 0; i < 8; ++i)
				{
					if (!((lanes >> i) & 1u)) continue;
					out[i] = child[i] ? cs.Hold(SDF::Stencil(cs.Ref(child[i]), cs.BorrowInputs ? NodeRef::Borrow(n.Mask.get()) : n.Mask,
						n.Mat, n.Negative)) : nullptr;
				}
				return;
			}
			case NodeKind::Flate:
			{
				uint32_t live = 0;
				float wide[8];
				for (int i = 0; i < 8; ++i)
				{
					wide[i] = radius[i];
					if (!((lanes >> i) & 1u)) continue;
					if (v[i] <= radius[i]) { live |= 1u << i; wide[i] = radius[i] + n.Threshold; }
					else out[i] = nullptr;
				}
				if (!live) return;
				const Node* child[8];
				ClipAt8(*n.Lhs, wide, live, child, ev, cs);
				for (int i = 0; i < 8; ++i)
					if ((live >> i) & 1u) out[i] = child[i] ? cs.Hold(SDF::Flate(cs.Ref(child[i]), n.Threshold)) : nullptr;
				return;
			}
			case NodeKind::Set:
			{
				uint32_t live = 0;
				for (int i = 0; i < 8; ++i)
				{
					if (!((lanes >> i) & 1u)) continue;
					if (v[i] <= radius[i]) live |= 1u << i;
					else out[i] = nullptr;
				}
				if (!live) return;
				const bool unionFamily = (n.Op == OpUnion || n.Op == OpBlendUnion);
				const bool diffFamily = (n.Op == OpDiff || n.Op == OpBlendDiff);
				uint32_t plain = live;     // lanes that go on to the clip at their own radius
				if (IsBlendOp(n.Op))
				{
					float wide[8];
					for (int i = 0; i < 8; ++i) wide[i] = radius[i] + n.Threshold;
					const Node* l[8];
					const Node* r[8];
					ClipAt8(*n.Lhs, wide, live, l, ev, cs);
					ClipAt8(*n.Rhs, wide, live, r, ev, cs);
					plain = 0;
					for (int i = 0; i < 8; ++i)
					{
						if (!((live >> i) & 1u)) continue;
						if (l[i] && r[i]) out[i] = RebuildSet(n, l[i], r[i], cs);
						else if (!unionFamily && !diffFamily) out[i] = nullptr;
						else plain |= 1u << i;
					}
					if (!plain) return;
				}
				const Node* l[8];
				const Node* r[8];
				ClipAt8(*n.Lhs, radius, plain, l, ev, cs);
				ClipAt8(*n.Rhs, radius, plain, r, ev, cs);
				for (int i = 0; i < 8; ++i)
				{
					if (!((plain >> i) & 1u)) continue;
					if (l[i] && r[i]) out[i] = RebuildSet(n, l[i], r[i], cs);
					else if (unionFamily) out[i] = l[i] ? l[i] : r[i];
					else if (diffFamily) out[i] = l[i];
					else out[i] = nullptr;
				}
				return;
			}
			}
		}
	}

	NodeRef Node::Clip(Vec3 p, float radius, bool borrow) const
	{
		PointEvaluations ev(p);
		ClipScratch cs(borrow);
		const Node* r = ClipAt(*this, radius, ev, cs);
		return r ? cs.Ref(r) : NodeRef();
	}

	void Node::Clip8(const Vec3 (&p)[8], const float (&radius)[8], NodeRef (&out)[8], bool borrow) const
	{
		Evaluations8 ev(p);
		ClipScratch cs(borrow);
		const Node* r[8];
		ClipAt8(*this, radius, 0xFFu, r, ev, cs);
		for (int i = 0; i < 8; ++i) out[i] = r[i] ? cs.Ref(r[i]) : NodeRef();
	}

	AABB Node::Bounds() const { return BoundsImpl(false); }
	AABB Node::InnerBounds() const { return BoundsImpl(true); }

	// Bounds / InnerBounds (sdf_evaluator.cpp:485-493, 622-630, 857-913, 1082-1096).
	AABB Node::BoundsImpl(bool inner) const
	{
		switch (Kind)
		{
		case NodeKind::Brush: return Xf.ApplyBounds(BrushBox);
		case NodeKind::Stencil: return Lhs->BoundsImpl(inner);
		case NodeKind::Flate:
		{
			AABB b = Lhs->BoundsImpl(inner);
			const float r2 = Threshold * 2.0f;
			b.Max = b.Max + Vec3(r2);
			b.Min = b.Min - Vec3(r2);
			return b;
		}
		case NodeKind::Set:
		{
			const AABB l = Lhs->BoundsImpl(inner), r = Rhs->BoundsImpl(inner);
			AABB c;
			if (Op == OpUnion || Op == OpBlendUnion) { c.Min = TernaryMin(l.Min, r.Min); c.Max = TernaryMax(l.Max, r.Max); }
			else if (Op == OpDiff || Op == OpBlendDiff) { c = l; }
			else { c.Min = TernaryMax(l.Min, r.Min); c.Max = TernaryMin(l.Max, r.Max); }
			if (IsBlendOp(Op) && !inner)
			{
				const Vec3 k(Threshold);
				const Vec3 limMin = TernaryMax(l.Min, r.Min) - k;
				const Vec3 limMax = TernaryMin(l.Max, r.Max) + k;
				c.Min = TernaryMin(c.Min, limMin);
				c.Max = TernaryMax(c.Max, limMax);
			}
			return c;
		}
		}
		return {};
	}

	void Node::Move(Vec3 by)
	{
		switch (Kind)
		{
		case NodeKind::Brush: Xf.Move(by); break;
		case NodeKind::Set: Lhs->Move(by); Rhs->Move(by); break;
		case NodeKind::Flate: Lhs->Move(by); break;
		case NodeKind::Stencil: Lhs->Move(by); Mask->Move(by); break;
		}
	}

	void Node::Rotate(Quat by)
	{
		switch (Kind)
		{
		case NodeKind::Brush: Xf.Rotate(by); break;
		case NodeKind::Set: Lhs->Rotate(by); Rhs->Rotate(by); break;
		case NodeKind::Flate: Lhs->Rotate(by); break;
		case NodeKind::Stencil: Lhs->Rotate(by); Mask->Rotate(by); break;
		}
	}

	// Set operators scale their blend threshold too; Flate keeps its radius
	// (sdf_evaluator.cpp:938-943, 1115-1118).
	void Node::Scale(float by)
	{
		switch (Kind)
		{
		case NodeKind::Brush: Xf.Scale(by); break;
		case NodeKind::Set: Threshold = Threshold * by; Lhs->Scale(by); Rhs->Scale(by); break;
		case NodeKind::Flate: Lhs->Scale(by); break;
		case NodeKind::Stencil: Lhs->Scale(by); Mask->Scale(by); break;
		}
	}

	// Paint only brushes without paint unless forced; stencils ignore it
	// (sdf_evaluator.cpp:524-530, 655-658, 945-949).
	void Node::ApplyMaterial(const MaterialRef& m, bool force)
	{
		switch (Kind)
		{
		case NodeKind::Brush: if (!Mat || force) Mat = m; break;
		case NodeKind::Set: Lhs->ApplyMaterial(m, force); Rhs->ApplyMaterial(m, force); break;
		case NodeKind::Flate: Lhs->ApplyMaterial(m, force); break;
		case NodeKind::Stencil: break;
		}
	}

	bool Node::HasPaint() const
	{
		switch (Kind)
		{
		case NodeKind::Brush: return Mat != nullptr;
		case NodeKind::Set: return Lhs->HasPaint() || Rhs->HasPaint();
		case NodeKind::Flate: return Lhs->HasPaint();
		case NodeKind::Stencil: return true;
		}
		return false;
	}

	bool Node::HasFiniteBounds() const
	{
		switch (Kind)
		{
		case NodeKind::Brush:
			for (int i = 0; i < 3; ++i)
				if (std::isinf(BrushBox.Min[i]) || std::isinf(BrushBox.Max[i])) return false;
			return true;
		case NodeKind::Set: return Lhs->HasFiniteBounds() || Rhs->HasFiniteBounds();
		default: return Lhs->HasFiniteBounds();
		}
	}

	int Node::LeafCount() const
	{
		switch (Kind)
		{
		case NodeKind::Brush: return 1;
		case NodeKind::Set: return Lhs->LeafCount() + Rhs->LeafCount();
		default: return Lhs->LeafCount();
		}
	}

	// Structural equality with material identity (sdf_evaluator.cpp:564-579, 696-709,
	// 1029-1037, 1150-1154).
	bool Node::Equals(const Node& o) const
	{
		if (this == &o) return true;
		if (Kind != o.Kind) return false;
		switch (Kind)
		{
		case NodeKind::Brush:
			if (Op != o.Op || Mat != o.Mat || !(Xf == o.Xf)) return false;
			for (int i = 0; i < BrushParamCount(Op); ++i)
				if (Params[i] != o.Params[i]) return false;
			return true;
		case NodeKind::Set:
			return Op == o.Op && Threshold == o.Threshold && Lhs->Equals(*o.Lhs) && Rhs->Equals(*o.Rhs);
		case NodeKind::Flate:
			return Threshold == o.Threshold && Lhs->Equals(*o.Lhs);
		case NodeKind::Stencil:
			return Negative == o.Negative && Mat == o.Mat && Lhs->Equals(*o.Lhs) && Mask->Equals(*o.Mask);
		}
		return false;
	}

	// Tetrahedral gradient with h = 1e-4, forward differences if it vanishes
	// (sdf_evaluator.cpp:298-333).
	Vec3 Node::Gradient(Vec3 p) const
	{
		const float h = 0.0001f;
		const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
		Vec3 g = xyy * Eval(p + xyy);
		g = g + yyx * Eval(p + yyx);
		g = g + yxy * Eval(p + yxy);
		g = g + xxx * Eval(p + xxx);
		const float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
		if (ls == 0.0f)
		{
			const float d = Eval(p);
			return Normalize(Vec3(Eval(p + xyy) - d, Eval(p + yxy) - d, Eval(p + yyx) - d));
		}
		return g / sqrtf(ls);
	}

	// GetMaterial (sdf_evaluator.cpp:537-547, 666-679, 957-1012, 1130-1133).
	const Material* Node::GetMaterial(Vec3 p) const
	{
		switch (Kind)
		{
		case NodeKind::Brush: return Mat.get();
		case NodeKind::Flate: return Lhs->GetMaterial(p);
		case NodeKind::Stencil:
		{
			const bool interior = Mask->Eval(p) < 0.0f;
			return interior == Negative ? Mat.get() : Lhs->GetMaterial(p);
		}
		case NodeKind::Set:
		{
			if (Op == OpDiff || Op == OpBlendDiff) return Lhs->GetMaterial(p);
			const float el = Lhs->Eval(p);
			const float er = Rhs->Eval(p);
			const float d = SetDistance(Op, el, er, Threshold);
			const bool takeLeft = IsBlendOp(Op) ? (fabsf(el - d) <= fabsf(er - d)) : (d == el);
			if (Op == OpUnion || Op == OpBlendUnion) return takeLeft ? Lhs->GetMaterial(p) : Rhs->GetMaterial(p);
			const Material* ml = Lhs->GetMaterial(p);
			const Material* mr = Rhs->GetMaterial(p);
			const bool lv = Lhs->HasPaint(), rv = Rhs->HasPaint();
			if (lv && rv) return takeLeft ? ml : mr;
			return lv ? ml : mr;
		}
		}
		return nullptr;
	}

	// SDFNode::RayMarch (sdf_evaluator.cpp:336-353).
	RayHit RayMarch(const Node& tree, Vec3 start, Vec3 dir, int max_iterations, float epsilon)
	{
		dir = Normalize(dir);
		Vec3 pos = start;
		float travel = 0.0f;
		for (int i = 0; i < max_iterations; ++i)
		{
			const float d = tree.Eval(pos);
			if (d <= epsilon) return { true, travel, pos };
			travel = travel + d;
			pos = dir * travel + start;
		}
		return { false, std::numeric_limits<float>::infinity(), pos };
	}

	namespace
	{
		NodeRef MakeBrush(uint32_t op, const float* params, AABB box, float a0 = 0.0f, float a1 = 0.0f, float a2 = 0.0f)
		{
			Node* n = new Node();
			n->Kind = NodeKind::Brush;
			n->Op = op;
			for (int i = 0; i < BrushParamCount(op); ++i) n->Params[i] = params[i];
			n->Args[0] = a0; n->Args[1] = a1; n->Args[2] = a2;
			n->BrushBox = box;
			n->StackSize = 1;
			return NodeRef(n);
		}

		AABB Symmetric(Vec3 h) { return { h * Vec3(-1.0f), h }; }
	}

	namespace SDF
	{
		NodeRef Sphere(float r) { const float p[1] = { r }; return MakeBrush(OpSphere, p, Symmetric(Vec3(r)), r); }
		NodeRef Ellipsoid(float x, float y, float z) { const float p[3] = { x, y, z }; return MakeBrush(OpEllipsoid, p, Symmetric(Vec3(x, y, z)), x, y, z); }
		NodeRef Box(float x, float y, float z) { const float p[3] = { x, y, z }; return MakeBrush(OpBox, p, Symmetric(Vec3(x, y, z)), x, y, z); }
		NodeRef Torus(float major, float minor)
		{
			const float p[2] = { major, minor };
			const float r = major + minor;
			return MakeBrush(OpTorus, p, Symmetric(Vec3(r, r, minor)), major, minor);
		}
		NodeRef Cylinder(float radius, float extent)
		{
			const float p[2] = { radius, extent };
			return MakeBrush(OpCylinder, p, Symmetric(Vec3(radius, radius, extent)), radius, extent);
		}
		// Unit normal; infinite bounds, halved when the normal is an axis (sdf_evaluator.cpp:1260-1294).
		NodeRef Plane(float nx, float ny, float nz)
		{
			const Vec3 n = Normalize(Vec3(nx, ny, nz));
			const float p[3] = { n.x, n.y, n.z };
			const float inf = std::numeric_limits<float>::infinity();
			AABB b = Symmetric(Vec3(inf));
			if (n.x == -1.0f) b.Min.x = 0.0f;
			else if (n.x == 1.0f) b.Max.x = 0.0f;
			else if (n.y == -1.0f) b.Min.y = 0.0f;
			else if (n.y == 1.0f) b.Max.y = 0.0f;
			else if (n.z == -1.0f) b.Min.z = 0.0f;
			else if (n.z == 1.0f) b.Max.z = 0.0f;
			return MakeBrush(OpPlane, p, b, nx, ny, nz);
		}
		NodeRef Cone(float radius, float height)
		{
			const float p[2] = { radius / height, height };
			return MakeBrush(OpCone, p, Symmetric(Vec3(radius, radius, (float)((double)height * 0.5))), radius, height);
		}
		NodeRef Coninder(float rl, float rh, float height)
		{
			const float half = (float)((double)height * 0.5);
			const float p[3] = { rl, rh, half };
			const float mr = fmaxf(rl, rh);
			return MakeBrush(OpConinder, p, Symmetric(Vec3(mr, mr, half)), rl, rh, height);
		}

		// Non-Diff operators put the operand with the deeper stack on the left
		// (sdf_evaluator.cpp:759-771); the stack need is max(L, R + 1).
		NodeRef MakeSet(uint32_t op, NodeRef lhs, NodeRef rhs, float k)
		{
			const bool diff = (op == OpDiff || op == OpBlendDiff);
			if (!diff && rhs->StackSize > lhs->StackSize) std::swap(lhs, rhs);
			Node* n = new Node();
			n->Kind = NodeKind::Set;
			n->Op = op;
			n->Threshold = k;
			n->StackSize = lhs->StackSize > rhs->StackSize + 1 ? lhs->StackSize : rhs->StackSize + 1;
			n->Lhs = std::move(lhs);
			n->Rhs = std::move(rhs);
			return NodeRef(n);
		}
		NodeRef Union(NodeRef l, NodeRef r) { return MakeSet(OpUnion, std::move(l), std::move(r), 0.0f); }
		NodeRef Diff(NodeRef l, NodeRef r) { return MakeSet(OpDiff, std::move(l), std::move(r), 0.0f); }
		NodeRef Inter(NodeRef l, NodeRef r) { return MakeSet(OpInter, std::move(l), std::move(r), 0.0f); }
		NodeRef BlendUnion(float k, NodeRef l, NodeRef r) { return MakeSet(OpBlendUnion, std::move(l), std::move(r), k); }
		NodeRef BlendDiff(float k, NodeRef l, NodeRef r) { return MakeSet(OpBlendDiff, std::move(l), std::move(r), k); }
		NodeRef BlendInter(float k, NodeRef l, NodeRef r) { return MakeSet(OpBlendInter, std::move(l), std::move(r), k); }

		NodeRef Flate(NodeRef node, float radius)
		{
			Node* n = new Node();
			n->Kind = NodeKind::Flate;
			n->StackSize = node->StackSize;
			n->Threshold = radius;
			n->Lhs = std::move(node);
			return NodeRef(n);
		}

		NodeRef Stencil(NodeRef node, NodeRef mask, MaterialRef material, bool negative)
		{
			Node* n = new Node();
			n->Kind = NodeKind::Stencil;
			n->StackSize = node->StackSize;
			n->Mat = std::move(material);
			n->Negative = negative;
			n->Lhs = std::move(node);
			n->Mask = std::move(mask);
			return NodeRef(n);
		}

		// Move the tree so the anchor point of its inner bounds sits at the origin;
		// anchors are in [-1, 1] per axis (sdf_evaluator.cpp:1171-1177).
		void Align(Node& tree, Vec3 anchors)
		{
			const Vec3 a = anchors * Vec3(0.5f) + Vec3(0.5f);
			const AABB b = tree.InnerBounds();
			const Vec3 mixed = b.Min * (Vec3(1.0f) - a) + b.Max * a;
			tree.Move(mixed * Vec3(-1.0f));
		}

		static void RotateAxis(Node& tree, int axis, float degrees)
		{
			const float r = (float)((double)(degrees * 0.01745329251994329576923690768489f) * .5);
			const float s = sinf(r), c = cosf(r);
			Quat q{ c, 0.0f, 0.0f, 0.0f };
			(&q.x)[axis] = s;
			tree.Rotate(q);
		}
		void RotateX(Node& tree, float degrees) { RotateAxis(tree, 0, degrees); }
		void RotateY(Node& tree, float degrees) { RotateAxis(tree, 1, degrees); }
		void RotateZ(Node& tree, float degrees) { RotateAxis(tree, 2, degrees); }
	}

	// Tree spec op codes (tangerine_gb300/workloads.py).
	namespace
	{
		enum SpecOp
		{
			SpecSphere = 1, SpecEllipsoid, SpecBox, SpecTorus, SpecCylinder, SpecPlane, SpecCone, SpecConinder,
			SpecUnion, SpecDiff, SpecInter, SpecBlendUnion, SpecBlendDiff, SpecBlendInter, SpecFlate,
			SpecMove, SpecRotate, SpecScale, SpecPaint, SpecAlign, SpecStencil, SpecTransform,
		};

		int SpecArity(int op)
		{
			switch (op)
			{
			case SpecSphere: return 1;
			case SpecEllipsoid: case SpecBox: case SpecPlane: case SpecConinder: return 3;
			case SpecTorus: case SpecCylinder: case SpecCone: return 2;
			case SpecUnion: case SpecDiff: case SpecInter: return 0;
			case SpecBlendUnion: case SpecBlendDiff: case SpecBlendInter: case SpecFlate: return 1;
			case SpecMove: case SpecPaint: case SpecAlign: return 3;
			case SpecRotate: case SpecStencil: return 4;
			case SpecScale: return 1;
			case SpecTransform: return 8;
			default: return -1;
			}
		}
	}

	NodeRef BuildFromSpec(const float* spec, int count, const char** error)
	{
		std::vector<NodeRef> stack;
		int i = 0;
		auto fail = [&](const char* why) { if (error) *error = why; return NodeRef(); };
		while (i < count)
		{
			const int op = (int)spec[i++];
			const int arity = SpecArity(op);
			if (arity < 0) return fail("unknown tree spec op");
			if (i + arity > count) return fail("truncated tree spec");
			const float* P = spec + i;
			i += arity;
			const size_t need = (op >= SpecUnion && op <= SpecBlendInter) || op == SpecStencil ? 2 :
				(op >= SpecFlate ? 1 : 0);
			if (stack.size() < need) return fail("tree spec stack underflow");
			switch (op)
			{
			case SpecSphere: stack.push_back(SDF::Sphere(P[0])); break;
			case SpecEllipsoid: stack.push_back(SDF::Ellipsoid(P[0], P[1], P[2])); break;
			case SpecBox: stack.push_back(SDF::Box(P[0], P[1], P[2])); break;
			case SpecTorus: stack.push_back(SDF::Torus(P[0], P[1])); break;
			case SpecCylinder: stack.push_back(SDF::Cylinder(P[0], P[1])); break;
			case SpecPlane: stack.push_back(SDF::Plane(P[0], P[1], P[2])); break;
			case SpecCone: stack.push_back(SDF::Cone(P[0], P[1])); break;
			case SpecConinder: stack.push_back(SDF::Coninder(P[0], P[1], P[2])); break;
			case SpecUnion: case SpecDiff: case SpecInter: case SpecBlendUnion: case SpecBlendDiff: case SpecBlendInter:
			{
				static const uint32_t map[] = { OpUnion, OpDiff, OpInter, OpBlendUnion, OpBlendDiff, OpBlendInter };
				NodeRef r = std::move(stack.back()); stack.pop_back();
				NodeRef l = std::move(stack.back()); stack.pop_back();
				stack.push_back(SDF::MakeSet(map[op - SpecUnion], std::move(l), std::move(r), op >= SpecBlendUnion ? P[0] : 0.0f));
				break;
			}
			case SpecFlate: stack.back() = SDF::Flate(std::move(stack.back()), P[0]); break;
			case SpecMove: stack.back()->Move(Vec3(P[0], P[1], P[2])); break;
			case SpecRotate: stack.back()->Rotate(Quat{ P[3], P[0], P[1], P[2] }); break;
			case SpecScale: stack.back()->Scale(P[0]); break;
			case SpecPaint:
			{
				auto m = std::make_shared<Material>();
				m->Rgb[0] = P[0]; m->Rgb[1] = P[1]; m->Rgb[2] = P[2];
				stack.back()->ApplyMaterial(m, false);
				break;
			}
			case SpecAlign: SDF::Align(*stack.back(), Vec3(P[0], P[1], P[2])); break;
			case SpecTransform:
			{
				// A brush's whole transform, set as it is: rotation (w x y z), translation, scale.
				Node& n = *stack.back();
				if (n.Kind != NodeKind::Brush) return fail("tree spec transform on a node that is not a brush");
				n.Xf.Rotation = Quat{ P[0], P[1], P[2], P[3] };
				n.Xf.Translation = Vec3(P[4], P[5], P[6]);
				n.Xf.Scalation = P[7];
				break;
			}
			case SpecStencil:
			{
				NodeRef mask = std::move(stack.back()); stack.pop_back();
				NodeRef node = std::move(stack.back()); stack.pop_back();
				auto m = std::make_shared<Material>();
				m->Rgb[0] = P[1]; m->Rgb[1] = P[2]; m->Rgb[2] = P[3];
				stack.push_back(SDF::Stencil(std::move(node), std::move(mask), m, P[0] != 0.0f));
				break;
			}
			}
		}
		if (stack.size() != 1) return fail("tree spec does not reduce to one tree");
		return std::move(stack.back());
	}

	void WriteSpec(const Node& n, std::vector<float>& out)
	{
		switch (n.Kind)
		{
		case NodeKind::Brush:
		{
			static const std::pair<uint32_t, int> brush[] = { { OpSphere, SpecSphere }, { OpEllipsoid, SpecEllipsoid },
				{ OpBox, SpecBox }, { OpTorus, SpecTorus }, { OpCylinder, SpecCylinder }, { OpPlane, SpecPlane },
				{ OpCone, SpecCone }, { OpConinder, SpecConinder } };
			int op = 0;
			for (const auto& b : brush) if (b.first == n.Op) op = b.second;
			out.push_back((float)op);
			for (int i = 0; i < SpecArity(op); ++i) out.push_back(n.Args[i]);
			const Transform& x = n.Xf;
			out.insert(out.end(), { (float)SpecTransform, x.Rotation.w, x.Rotation.x, x.Rotation.y, x.Rotation.z,
				x.Translation.x, x.Translation.y, x.Translation.z, x.Scalation });
			if (n.Mat) out.insert(out.end(), { (float)SpecPaint, n.Mat->Rgb[0], n.Mat->Rgb[1], n.Mat->Rgb[2] });
			break;
		}
		case NodeKind::Set:
		{
			WriteSpec(*n.Lhs, out);
			WriteSpec(*n.Rhs, out);
			static const std::pair<uint32_t, int> set[] = { { OpUnion, SpecUnion }, { OpDiff, SpecDiff }, { OpInter, SpecInter },
				{ OpBlendUnion, SpecBlendUnion }, { OpBlendDiff, SpecBlendDiff }, { OpBlendInter, SpecBlendInter } };
			int op = 0;
			for (const auto& b : set) if (b.first == n.Op) op = b.second;
			out.push_back((float)op);
			if (op >= SpecBlendUnion) out.push_back(n.Threshold);
			break;
		}
		case NodeKind::Flate:
			WriteSpec(*n.Lhs, out);
			out.insert(out.end(), { (float)SpecFlate, n.Threshold });
			break;
		case NodeKind::Stencil:
			WriteSpec(*n.Lhs, out);
			WriteSpec(*n.Mask, out);
			out.insert(out.end(), { (float)SpecStencil, n.Negative ? 1.0f : 0.0f, n.Mat ? n.Mat->Rgb[0] : 1.0f,
				n.Mat ? n.Mat->Rgb[1] : 1.0f, n.Mat ? n.Mat->Rgb[2] : 1.0f });
			break;
		}
	}

	NodeRef CopyTree(const Node& n)
	{
		switch (n.Kind)
		{
		case NodeKind::Brush:
		{
			Node* c = new Node();
			c->Kind = NodeKind::Brush;
			c->Op = n.Op;
			c->StackSize = n.StackSize;
			for (int i = 0; i < 3; ++i) { c->Params[i] = n.Params[i]; c->Args[i] = n.Args[i]; }
			c->BrushBox = n.BrushBox;
			c->Xf = n.Xf;
			c->Mat = n.Mat;
			return NodeRef(c);
		}
		case NodeKind::Set: return SDF::MakeSet(n.Op, CopyTree(*n.Lhs), CopyTree(*n.Rhs), n.Threshold);
		case NodeKind::Flate: return SDF::Flate(CopyTree(*n.Lhs), n.Threshold);
		case NodeKind::Stencil: return SDF::Stencil(CopyTree(*n.Lhs), CopyTree(*n.Mask), n.Mat, n.Negative);
		}
		return NodeRef();
	}
}
