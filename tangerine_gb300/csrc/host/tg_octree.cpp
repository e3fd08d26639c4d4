// Export octree construction and compilation of each octree cell's clipped subtree into
// the GPU record format (tg_layout.hpp).
#include "tg_octree.hpp"
#include "tg_pool.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>
#include <memory>
#include <unordered_map>

namespace tg
{
	namespace
	{
		struct TmpCell
		{
			AABB Bounds;
			Vec3 Pivot;
			float Radius = 0.0f;
			bool Terminus = false;
			bool Incomplete = false;
			bool ClippedAway = false;   // the clip to this cell's sphere returned null
			bool Expanded = false;      // split into eight children
			uint32_t NullOctants = 0;   // children whose clip returned null
			int Leaves = 0;
			NodeRef Eval;
			TmpCell* Kids[8] = { nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr };
		};

		// The build's cells, a block per level.  A cell dropped from the tree is only
		// unlinked: its clipped tree is released with the blocks, on the background thread,
		// after the build (the live cells' trees borrow only from live ancestors).
		struct CellArena
		{
			std::vector<std::unique_ptr<TmpCell[]>> Blocks;
			TmpCell* Take(size_t n)
			{
				Blocks.emplace_back(new TmpCell[n]);
				return Blocks.back().get();
			}
			void ReleaseLater()
			{
				auto held = std::make_shared<std::vector<std::unique_ptr<TmpCell[]>>>(std::move(Blocks));
				WorkerPool::Get().Later([held]() { held->clear(); });
			}
		};

		struct BuildParams
		{
			float Target;
			bool Coalesce;
			int MaxDepth;
		};

		// SDFOctree ctor (sdf_evaluator.cpp:1641-1700): the cell's pivot is its min corner
		// plus half the longest side; its evaluator is the parent's clipped to the sphere
		// through the cube's corners.
		void PlaceCell(TmpCell& c, float& span)
		{
			const Vec3 e = c.Bounds.Max - c.Bounds.Min;
			span = fmaxf(fmaxf(e.x, e.y), e.z);
			const float half = (float)((double)span * 0.5);
			c.Pivot = Vec3(half) + c.Bounds.Min;
			c.Radius = (float)((double)Length(Vec3(span)) * 0.5);
		}

		void SetEvaluator(TmpCell& c, NodeRef eval, float span, const BuildParams& bp)
		{
			c.Eval = std::move(eval);
			c.ClippedAway = !c.Eval;
			c.Leaves = c.Eval ? c.Eval->LeafCount() : 0;
			c.Terminus = span <= bp.Target || !c.Eval;
			c.Incomplete = !c.Terminus;
		}

		void InitCell(TmpCell& c, const NodeRef& in, const BuildParams& bp)
		{
			float span;
			PlaceCell(c, span);
			SetEvaluator(c, in->Clip(c.Pivot, c.Radius, true), span, bp);
		}

		// The eight children of an expanded cell, their clips sharing one walk of its tree.
		void InitChildren(TmpCell& parent, const BuildParams& bp)
		{
			Vec3 pivots[8];
			float radii[8], spans[8];
			for (int i = 0; i < 8; ++i)
			{
				PlaceCell(*parent.Kids[i], spans[i]);
				pivots[i] = parent.Kids[i]->Pivot;
				radii[i] = parent.Kids[i]->Radius;
			}
			NodeRef evals[8];
			parent.Eval->Clip8(pivots, radii, evals, true);
			for (int i = 0; i < 8; ++i) SetEvaluator(*parent.Kids[i], std::move(evals[i]), spans[i], bp);
		}

		// One child of an expanded cell on its own (Clip to its sphere): the same evaluator
		// InitChildren gives it, for levels with too few cells to keep the workers busy.
		void InitChild(TmpCell& parent, int i, const BuildParams& bp)
		{
			TmpCell& kid = *parent.Kids[i];
			float span;
			PlaceCell(kid, span);
			SetEvaluator(kid, parent.Eval->Clip(kid.Pivot, kid.Radius, true), span, bp);
		}

		// The tail of SDFOctree::Populate (sdf_evaluator.cpp:1703-1783), once the children
		// exist and are final themselves: drop empty children, shrink the bounds to the live
		// ones, and merge the children back into this cell when they all ended and share
		// one evaluator, or when few brushes remain.
		void FinishCell(TmpCell& c, const BuildParams& bp, int depth)
		{
			bool uniform = true, penultimate = true;
			int live = 0;
			for (int i = 0; i < 8; ++i)
			{
				if (!c.Kids[i]->Eval)
				{
					if (c.Kids[i]->ClippedAway) c.NullOctants |= 1u << i;
					c.Kids[i] = nullptr;
					continue;
				}
				uniform = uniform && c.Eval->Equals(*c.Kids[i]->Eval);
				penultimate = penultimate && c.Kids[i]->Terminus;
				if (live == 0)
				{
					c.Bounds = c.Kids[i]->Bounds;
				}
				else
				{
					c.Bounds.Min = TernaryMin(c.Bounds.Min, c.Kids[i]->Bounds.Min);
					c.Bounds.Max = TernaryMax(c.Bounds.Max, c.Kids[i]->Bounds.Max);
				}
				++live;
			}
			if (live == 0)
			{
				c.Eval = NodeRef();
				c.Terminus = true;
				return;
			}
			const int limit = depth > 3 ? depth : 3;
			if (bp.Coalesce && ((penultimate && uniform) || c.Leaves <= limit))
			{
				for (auto& k : c.Kids) k = nullptr;
				c.Terminus = true;
			}
		}

		// SDFOctree::Populate's recursion, level by level: every cell of a level is clipped
		// in parallel (the clips are independent), then the cells that go on split into
		// eight children for the next level.  The merge decisions run afterwards, bottom up
		// a level at a time; they depend only on a cell's descendants, so the octree is the one the reference's depth-first recursion
		// builds.  `tops` are disjoint subtrees, all at top_depth.
		void BuildLevels(const std::vector<TmpCell*>& tops, const BuildParams& bp, int top_depth, CellArena& arena)
		{
			std::vector<TmpCell*> level = tops;
			std::vector<std::vector<TmpCell*>> expanded;   // per depth from top_depth
			int depth = top_depth;
			while (!level.empty())
			{
				std::vector<TmpCell*> parents;
				for (TmpCell* c : level)
				{
					if (c->Terminus) continue;
					if (!(bp.Coalesce || bp.MaxDepth == -1 || depth < bp.MaxDepth)) continue;
					c->Incomplete = false;
					c->Expanded = true;
					parents.push_back(c);
				}
				if (parents.empty()) break;
				TmpCell* kids = arena.Take(parents.size() * 8);
				for (size_t p = 0; p < parents.size(); ++p)
				{
					TmpCell* c = parents[p];
					for (int i = 0; i < 8; ++i)
					{
						AABB b = c->Bounds;
						if (i & 1) b.Min.x = c->Pivot.x; else b.Max.x = c->Pivot.x;
						if (i & 2) b.Min.y = c->Pivot.y; else b.Max.y = c->Pivot.y;
						if (i & 4) b.Min.z = c->Pivot.z; else b.Max.z = c->Pivot.z;
						c->Kids[i] = kids + p * 8 + i;
						c->Kids[i]->Bounds = b;
					}
				}
				// The clips are handed out largest tree first (leaf count), so that no long one
				// starts last; each writes only its own parent's children.
				WorkerPool& pool = WorkerPool::Get();
				std::vector<int> order(parents.size());
				for (size_t j = 0; j < order.size(); ++j) order[j] = (int)j;
				std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return parents[(size_t)a]->Leaves > parents[(size_t)b]->Leaves; });
				if ((int)parents.size() <= pool.Workers())
					pool.ParallelFor((int)parents.size() * 8, [&](int j) { InitChild(*parents[(size_t)order[(size_t)(j / 8)]], j % 8, bp); });
				else
					pool.ParallelFor((int)parents.size(), [&](int j) { InitChildren(*parents[(size_t)order[(size_t)j]], bp); });
				level.clear();
				for (TmpCell* c : parents)
					for (TmpCell* k : c->Kids) level.push_back(k);
				expanded.push_back(std::move(parents));
				++depth;
			}
			for (size_t d = expanded.size(); d-- > 0;)
				for (TmpCell* c : expanded[d]) FinishCell(*c, bp, top_depth + (int)d);
		}

		// SDFOctree::Walk's incomplete search (sodapop.cpp:108-124): cells that were never
		// split because the depth limit stopped them.
		void FindIncomplete(TmpCell& c, std::vector<TmpCell*>& out)
		{
			if (c.Terminus || c.Incomplete)
			{
				if (c.Incomplete) out.push_back(&c);
				return;
			}
			for (TmpCell* k : c.Kids)
				if (k) FindIncomplete(*k, out);
		}

		size_t CountCells(const TmpCell& t)
		{
			size_t n = 1;
			if (!t.Terminus)
				for (const TmpCell* k : t.Kids)
					if (k) n += CountCells(*k);
			return n;
		}

		void Flatten(TmpCell& t, std::vector<Octree::Cell>& out)
		{
			const int index = (int)out.size();
			out.emplace_back();
			{
				Octree::Cell& c = out.back();
				c.Bounds = t.Bounds;
				c.Pivot = t.Pivot;
				c.ClipRadius = t.Radius;
				c.NullOctants = t.NullOctants;
				c.Terminus = t.Terminus;
				c.Incomplete = t.Incomplete;
				c.EvaluatorLeaves = t.Leaves;
				c.Evaluator = std::move(t.Eval);   // the build is done with it
			}
			if (t.Terminus) return;
			for (int i = 0; i < 8; ++i)
			{
				if (t.Kids[i])
				{
					const int child = (int)out.size();
					Flatten(*t.Kids[i], out);
					out[index].Children[i] = child;
				}
			}
		}
	}

	bool Octree::Build(const NodeRef& root, float target, bool coalesce, int max_depth, const RootSeen* on_root)
	{
		Cells.clear();
		if (!root || !root->HasFiniteBounds()) return false;
		// Bounds().BoundingCube() + 0 margin (sdf_evaluator.cpp:1616).
		AABB cube = root->Bounds().BoundingCube();
		if (!cube.Degenerate())
		{
			cube.Min = cube.Min - Vec3(0.0f);
			cube.Max = cube.Max + Vec3(0.0f);
		}
		if (cube.Volume() == 0.0f) return false;
		BuildParams bp{ target, coalesce, max_depth };
		CellArena arena;
		TmpCell* top = arena.Take(1);
		top->Bounds = cube;
		InitCell(*top, root, bp);
		if (!top->Eval) return false;
		// The levels below change the root's bounds but not its pivot, clip radius or
		// evaluator (FinishCell only drops the evaluator when every octant is empty, and
		// then the build fails).
		if (on_root && *on_root) (*on_root)(top->Pivot, top->Radius, top->Eval);
		BuildLevels({ top }, bp, 1, arena);
		// SDFOctree::Create returns nullptr when the root lost its evaluator while
		// populating (every octant clipped away).
		if (!top->Eval)
		{
			arena.ReleaseLater();
			return false;
		}
		Cells.reserve(CountCells(*top));
		Flatten(*top, Cells);
		arena.ReleaseLater();
		return true;
	}

	bool Octree::BuildMeshing(const NodeRef& root)
	{
		Cells.clear();
		if (!root || !root->HasFiniteBounds()) return false;
		AABB cube = root->Bounds().BoundingCube();
		if (!cube.Degenerate())
		{
			cube.Min = cube.Min - Vec3(0.0f);
			cube.Max = cube.Max + Vec3(0.0f);
		}
		if (cube.Volume() == 0.0f) return false;
		const BuildParams first{ 0.25f, false, 3 };
		CellArena arena;
		TmpCell* top = arena.Take(1);
		top->Bounds = cube;
		InitCell(*top, root, first);
		if (!top->Eval) return false;
		BuildLevels({ top }, first, 1, arena);
		if (!top->Eval)
		{
			arena.ReleaseLater();
			return false;
		}
		// Populate(false, 3, -1) of each incomplete cell: its children start at depth 4 and
		// split without limit.  The cells are disjoint, so one level-parallel pass serves
		// them all.
		std::vector<TmpCell*> incomplete;
		FindIncomplete(*top, incomplete);
		const BuildParams second{ 0.25f, false, -1 };
		BuildLevels(incomplete, second, 3, arena);
		Cells.reserve(CountCells(*top));
		Flatten(*top, Cells);
		arena.ReleaseLater();
		return true;
	}

	// The deepest cell on the point's path that has an evaluator: a child whose own search
	// finds none hands the point back to its parent.
	int Octree::Descend(Vec3 p) const
	{
		int at = 0, found = Cells[0].Evaluator ? 0 : -1;
		for (;;)
		{
			const Cell& c = Cells[at];
			if (c.Evaluator) found = at;
			if (c.Terminus) return found;
			int i = 0;
			if (p.x > c.Pivot.x) i |= 1;
			if (p.y > c.Pivot.y) i |= 2;
			if (p.z > c.Pivot.z) i |= 4;
			if (c.Children[i] < 0) return found;
			at = c.Children[i];
		}
	}

	namespace
	{
		void PushWord(std::vector<uint32_t>& w, float f) { w.push_back(FloatBits(f)); }

		// SDFNode::Compile (sdf_evaluator.cpp:409-429, 495-507, 632-635, 915-924, 1098-1103).
		void ReferenceWords(const Node& n, std::vector<uint32_t>& w)
		{
			switch (n.Kind)
			{
			case NodeKind::Brush:
			{
				const Transform& t = n.Xf;
				const bool rot = !t.Rotation.IsIdentity();
				const bool scl = t.Scalation != 1.0f;
				const bool trn = !(t.Translation.x == 0.0f && t.Translation.y == 0.0f && t.Translation.z == 0.0f);
				if (rot || scl)
				{
					const Mat4 inv = MatInverse(t.ToMatrix());
					w.push_back(OpMatrix);
					for (float v : inv.m) PushWord(w, v);
				}
				else if (trn)
				{
					w.push_back(OpOffset);
					PushWord(w, -t.Translation.x); PushWord(w, -t.Translation.y); PushWord(w, -t.Translation.z);
				}
				w.push_back(n.Op);
				for (int i = 0; i < BrushParamCount(n.Op); ++i) PushWord(w, n.Params[i]);
				if (scl)
				{
					w.push_back(OpScaleField);
					PushWord(w, t.Scalation);
				}
				break;
			}
			case NodeKind::Set:
				ReferenceWords(*n.Lhs, w);
				ReferenceWords(*n.Rhs, w);
				w.push_back(n.Op);
				if (IsBlendOp(n.Op)) PushWord(w, n.Threshold);
				break;
			case NodeKind::Flate:
				ReferenceWords(*n.Lhs, w);
				w.push_back(OpFlate);
				PushWord(w, n.Threshold);
				break;
			case NodeKind::Stencil:
				ReferenceWords(*n.Lhs, w);
				break;
			}
		}

		// Facts the emitter caches per node: the slot of a brush's records and whether a
		// subtree has paint.  Open addressing on the node's address; one table per emitter,
		// so emitters on different threads share nothing.
		class NodeFacts
		{
		public:
			struct Entry
			{
				const Node* Key;
				int32_t Record;     // -1: not built
				int8_t Paint;       // -1: not known
				int32_t SurfQuads;  // -1: not known; else the surface program's quads
				int32_t SurfPeak;   // and the stack depth it reaches
			};
			NodeFacts() { Slots.assign(1024, Entry{ nullptr, -1, -1, -1, 0 }); }
			// The entry of n, or null (no insertion).
			const Entry* Find(const Node* n) const
			{
				const size_t mask = Slots.size() - 1;
				for (size_t i = Hash(n) & mask;; i = (i + 1) & mask)
				{
					const Entry& e = Slots[i];
					if (e.Key == n) return &e;
					if (!e.Key) return nullptr;
				}
			}
			// The entry of n, created if absent; valid until the next call.
			Entry& At(const Node* n)
			{
				if ((Size + 1) * 2 > Slots.size()) Grow();
				const size_t mask = Slots.size() - 1;
				size_t i = Hash(n) & mask;
				for (;;)
				{
					Entry& e = Slots[i];
					if (e.Key == n) return e;
					if (!e.Key)
					{
						e = Entry{ n, -1, -1, -1, 0 };
						++Size;
						return e;
					}
					i = (i + 1) & mask;
				}
			}

		private:
			static size_t Hash(const Node* n)
			{
				uint64_t x = (uint64_t)(uintptr_t)n;
				x ^= x >> 33;
				x *= 0xff51afd7ed558ccdULL;
				x ^= x >> 33;
				return (size_t)x;
			}
			void Grow()
			{
				std::vector<Entry> old;
				old.swap(Slots);
				Slots.assign(old.size() * 2, Entry{ nullptr, -1, -1, -1, 0 });
				Size = 0;
				for (const Entry& e : old)
				{
					if (!e.Key) continue;
					Entry& n = At(e.Key);
					n.Record = e.Record;
					n.Paint = e.Paint;
					n.SurfQuads = e.SurfQuads;
					n.SurfPeak = e.SurfPeak;
				}
			}
			std::vector<Entry> Slots;
			size_t Size = 0;
		};

		// Emits record programs.  Clipped trees share their brush nodes with the full tree,
		// so one brush appears in many cells' programs: its records (an inverse matrix is
		// ~200 flops to build) and every subtree's paint flag are computed once per emitter.
		// A brush's two records, as spans of a record arena.
		struct RecordSpans
		{
			int DistanceAt, DistanceFloats, SurfaceAt, SurfaceFloats;
		};

		struct Emitter
		{
			std::vector<float>& Code;
			const std::unordered_map<const Material*, int>& Materials;
			std::vector<float> Arena;                    // this emitter's own brush records
			std::vector<RecordSpans> Spans;
			const Emitter* Shared = nullptr;             // records built before the parallel emission
			bool NonLipschitz = false;
			NodeFacts Facts;

			Emitter(std::vector<float>& code, const std::unordered_map<const Material*, int>& materials, const Emitter* shared = nullptr)
				: Code(code), Materials(materials), Shared(shared) {}

			void Quad(uint32_t head, float a, float b, float c)
			{
				Code.push_back(BitsFloat(head));
				Code.push_back(a);
				Code.push_back(b);
				Code.push_back(c);
			}
			int MaterialIndex(const Material* m) const
			{
				if (!m) return -1;
				auto it = Materials.find(m);
				return it == Materials.end() ? -1 : it->second;
			}
			bool HasPaint(const Node& n)
			{
				{
					const NodeFacts::Entry& e = Facts.At(&n);
					if (e.Paint >= 0) return e.Paint != 0;
				}
				bool paint = false;
				switch (n.Kind)
				{
				case NodeKind::Brush: paint = n.Mat != nullptr; break;
				case NodeKind::Set: paint = HasPaint(*n.Lhs) || HasPaint(*n.Rhs); break;
				case NodeKind::Flate: paint = HasPaint(*n.Lhs); break;
				case NodeKind::Stencil: paint = true; break;
				}
				Facts.At(&n).Paint = paint ? 1 : 0;
				return paint;
			}

			// Records of one brush: [distance quads, surface quads], built once per emitter
			// (or taken from the shared emitter's arena).
			// The arena holding a brush's records and their spans there.
			void SpansOf(const Node& n, const float*& arena, const RecordSpans*& sp)
			{
				const NodeFacts::Entry* shared = Shared ? Shared->Facts.Find(&n) : nullptr;
				if (shared && shared->Record >= 0)
				{
					arena = Shared->Arena.data();
					sp = &Shared->Spans[(size_t)shared->Record];
				}
				else
				{
					const int r = Records(n);
					arena = Arena.data();
					sp = &Spans[(size_t)r];
				}
			}

			void AppendRecords(const Node& n, bool surface)
			{
				const float* arena;
				const RecordSpans* sp;
				SpansOf(n, arena, sp);
				const float* from = arena + (surface ? sp->SurfaceAt : sp->DistanceAt);
				(surface ? LastSurfaceBrushAt : LastBrushAt) = Code.size();
				Code.insert(Code.end(), from, from + (surface ? sp->SurfaceFloats : sp->DistanceFloats));
			}
			size_t LastBrushAt = 0;         // float index of the last distance brush record's head
			size_t LastSurfaceBrushAt = 0;  // and of the last surface brush record's

			// A brush's two records: its distance quads (at most 5), then its surface quads (4).
			struct BrushRecords
			{
				float Data[36];
				int DistanceFloats, SurfaceFloats;
			};

			// The records of brush n.  Touches no table of the emitter: safe on any thread.
			void MakeRecords(const Node& n, BrushRecords& out) const
			{
				int k = 0;
				auto put = [&](float a, float b, float c, float d)
				{
					out.Data[k] = a; out.Data[k + 1] = b; out.Data[k + 2] = c; out.Data[k + 3] = d;
					k += 4;
				};
				const Transform& t = n.Xf;
				const bool rot = !t.Rotation.IsIdentity();
				const bool scl = t.Scalation != 1.0f;
				const bool trn = !(t.Translation.x == 0.0f && t.Translation.y == 0.0f && t.Translation.z == 0.0f);
				uint32_t flags = 0;
				if (rot || scl) flags |= RecMatrix;
				else if (trn) flags |= RecOffset;
				if (scl) flags |= RecScale;
				put(BitsFloat(n.Op | flags), n.Params[0], n.Params[1], n.Params[2]);
				if (flags & RecMatrix)
				{
					const Mat4 inv = MatInverse(t.ToMatrix());
					// Row r of the 3x4 affine part: (m[0][r], m[1][r], m[2][r], m[3][r]).
					for (int r = 0; r < 3; ++r) put(inv.at(0, r), inv.at(1, r), inv.at(2, r), inv.at(3, r));
				}
				else if (flags & RecOffset)
				{
					put(-t.Translation.x, -t.Translation.y, -t.Translation.z, 0.0f);
				}
				if (flags & RecScale) put(t.Scalation, 0.0f, 0.0f, 0.0f);
				out.DistanceFloats = k;
				const Quat qi = Inverse(t.Rotation);
				put(BitsFloat(n.Op), n.Params[0], n.Params[1], n.Params[2]);
				put(qi.w, qi.x, qi.y, qi.z);
				put(t.Translation.x, t.Translation.y, t.Translation.z, t.Scalation);
				put(BitsFloat((uint32_t)MaterialIndex(n.Mat.get())), 0.0f, 0.0f, 0.0f);
				out.SurfaceFloats = k - out.DistanceFloats;
			}

			// Appends brush n's records to this emitter's arena; returns their slot.
			int AddRecords(const Node& n, const BrushRecords& r)
			{
				const int32_t slot = (int32_t)Spans.size();
				RecordSpans sp;
				sp.DistanceAt = (int)Arena.size();
				sp.DistanceFloats = r.DistanceFloats;
				sp.SurfaceAt = sp.DistanceAt + r.DistanceFloats;
				sp.SurfaceFloats = r.SurfaceFloats;
				Arena.insert(Arena.end(), r.Data, r.Data + r.DistanceFloats + r.SurfaceFloats);
				Spans.push_back(sp);
				Facts.At(&n).Record = slot;
				return slot;
			}

			int Records(const Node& n)
			{
				{
					const NodeFacts::Entry& e = Facts.At(&n);
					if (e.Record >= 0) return e.Record;
				}
				BrushRecords r;
				MakeRecords(n, r);
				return AddRecords(n, r);
			}

			// Each brush under n once, depth first (a brush being collected has Record -2).
			void CollectBrushes(const Node& n, std::vector<const Node*>& out)
			{
				switch (n.Kind)
				{
				case NodeKind::Brush:
				{
					NodeFacts::Entry& e = Facts.At(&n);
					if (e.Record == -1)
					{
						e.Record = -2;
						out.push_back(&n);
					}
					break;
				}
				case NodeKind::Set: CollectBrushes(*n.Lhs, out); CollectBrushes(*n.Rhs, out); break;
				case NodeKind::Flate: CollectBrushes(*n.Lhs, out); break;
				case NodeKind::Stencil: CollectBrushes(*n.Lhs, out); CollectBrushes(*n.Mask, out); break;
				}
			}

			// Builds the records of every brush under n (the full tree, before emission): the
			// brushes' records are computed on the worker pool, then appended in depth-first
			// order.
			void BuildAllRecords(const Node& n)
			{
				std::vector<const Node*> brushes;
				CollectBrushes(n, brushes);
				std::vector<BrushRecords> built(brushes.size());
				WorkerPool::Get().ParallelFor((int)brushes.size(), [&](int i) { MakeRecords(*brushes[(size_t)i], built[(size_t)i]); });
				Arena.reserve(Arena.size() + brushes.size() * 36);
				Spans.reserve(Spans.size() + brushes.size());
				for (size_t i = 0; i < brushes.size(); ++i) AddRecords(*brushes[i], built[i]);
			}

			// Distance program: Tangerine's postfix program with each brush's transform,
			// primitive and field scale fused into one record.  Returns the deepest stack the
			// program reaches (accumulator + spilled operands) counting every brush as a push,
			// fused or not: a set holds its left operand while its right one runs.
			int Distance(const Node& n)
			{
				switch (n.Kind)
				{
				case NodeKind::Brush:
					if (n.Op == OpEllipsoid) NonLipschitz = true;
					AppendRecords(n, false);
					return 1;
				case NodeKind::Set:
				{
					const int l = Distance(*n.Lhs);
					const int r = Distance(*n.Rhs);
					// A brush right operand (the usual case: the tree leans left) is combined
					// with the left operand in the brush's own step, without a stack push.
					if (n.Rhs->Kind == NodeKind::Brush)
						Code[LastBrushAt] = BitsFloat(FloatBits(Code[LastBrushAt]) | RecThenSet);
					Quad(n.Op, IsBlendOp(n.Op) ? n.Threshold : 0.0f, 0.0f, 0.0f);
					return l > r + 1 ? l : r + 1;
				}
				case NodeKind::Flate:
				{
					const int d = Distance(*n.Lhs);
					Quad(OpFlate, n.Threshold, 0.0f, 0.0f);
					return d;
				}
				case NodeKind::Stencil:
					return Distance(*n.Lhs);
				}
				return 0;
			}

			// The quads Surface(n) emits and the deepest stack its program reaches (every
			// brush a push, every set and stencil end a pop), without emitting it: both depend
			// on the subtree alone, so they are kept per node (the shared emitter's table first).
			void SurfaceSize(const Node& n, int& quads, int& peak)
			{
				const NodeFacts::Entry* known = Shared ? Shared->Facts.Find(&n) : nullptr;
				if (!(known && known->SurfQuads >= 0)) known = Facts.Find(&n);
				if (known && known->SurfQuads >= 0)
				{
					quads = known->SurfQuads;
					peak = known->SurfPeak;
					return;
				}
				int q = 0, p = 0;
				switch (n.Kind)
				{
				case NodeKind::Brush:
				{
					const float* arena;
					const RecordSpans* sp;
					SpansOf(n, arena, sp);
					q = sp->SurfaceFloats / 4;
					p = 1;
					break;
				}
				case NodeKind::Set:
				{
					int ql, pl, qr, pr;
					SurfaceSize(*n.Lhs, ql, pl);
					SurfaceSize(*n.Rhs, qr, pr);
					q = ql + qr + 1;
					p = pl > pr + 1 ? pl : pr + 1;
					break;
				}
				case NodeKind::Flate:
					SurfaceSize(*n.Lhs, q, p);
					q += 1;
					break;
				case NodeKind::Stencil:
				{
					int ql, pl, qm, pm;
					SurfaceSize(*n.Lhs, ql, pl);
					SurfaceSize(*n.Mask, qm, pm);
					q = ql + 1 + qm + 1;
					p = pl > pm + 1 ? pl : pm + 1;
					break;
				}
				}
				NodeFacts::Entry& e = Facts.At(&n);
				e.SurfQuads = q;
				e.SurfPeak = p;
				quads = q;
				peak = p;
			}

			// Surface program: the subtree as SDFNode::Eval / GetMaterial walk it.
			// Returns the deepest stack the program reaches, counted as SurfaceSize counts it.
			int Surface(const Node& n)
			{
				switch (n.Kind)
				{
				case NodeKind::Brush:
					AppendRecords(n, true);
					return 1;
				case NodeKind::Set:
				{
					const int l = Surface(*n.Lhs);
					const int r = Surface(*n.Rhs);
					uint32_t flags = 0;
					if (HasPaint(*n.Lhs)) flags |= RecLhsPaint;
					if (HasPaint(*n.Rhs)) flags |= RecRhsPaint;
					if (n.Rhs->Kind == NodeKind::Brush)
						Code[LastSurfaceBrushAt] = BitsFloat(FloatBits(Code[LastSurfaceBrushAt]) | RecThenSet);
					Quad(n.Op | flags, n.Threshold, 0.0f, 0.0f);
					return l > r + 1 ? l : r + 1;
				}
				case NodeKind::Flate:
				{
					const int d = Surface(*n.Lhs);
					Quad(OpFlate, n.Threshold, 0.0f, 0.0f);
					return d;
				}
				case NodeKind::Stencil:
				{
					const int l = Surface(*n.Lhs);
					const size_t begin = Code.size();
					Quad(OpMaskBegin, 0.0f, 0.0f, 0.0f);
					const int m = Surface(*n.Mask);
					Quad(OpStencilEnd | (n.Negative ? RecNegative : 0u), BitsFloat((uint32_t)MaterialIndex(n.Mat.get())), 0.0f, 0.0f);
					// Quads to skip after the MaskBegin record when only distances are needed.
					const int skip = (int)((Code.size() - begin) / 4) - 1;
					Code[begin + 1] = BitsFloat((uint32_t)skip);
					return l > m + 1 ? l : m + 1;
				}
				}
				return 0;
			}
		};

		// Material indices in depth-first order of the full tree: every clipped tree shares
		// its brushes (and their materials) with it.
		void CollectMaterials(const Node& n, std::unordered_map<const Material*, int>& index, std::vector<const Material*>& list)
		{
			auto add = [&](const Material* m)
			{
				if (m && index.emplace(m, (int)list.size()).second) list.push_back(m);
			};
			switch (n.Kind)
			{
			case NodeKind::Brush: add(n.Mat.get()); break;
			case NodeKind::Set: CollectMaterials(*n.Lhs, index, list); CollectMaterials(*n.Rhs, index, list); break;
			case NodeKind::Flate: CollectMaterials(*n.Lhs, index, list); break;
			case NodeKind::Stencil:
				CollectMaterials(*n.Lhs, index, list);
				CollectMaterials(*n.Mask, index, list);
				add(n.Mat.get());
				break;
			}
		}

	}

	// Ellipsoid distances are a bound estimate, not 1-Lipschitz; every other primitive and
	// every set operator here is.
	bool HasNonLipschitzBrush(const Node& n)
	{
		switch (n.Kind)
		{
		case NodeKind::Brush: return n.Op == OpEllipsoid;
		case NodeKind::Set: return HasNonLipschitzBrush(*n.Lhs) || HasNonLipschitzBrush(*n.Rhs);
		case NodeKind::Flate: return HasNonLipschitzBrush(*n.Lhs);
		case NodeKind::Stencil: return HasNonLipschitzBrush(*n.Lhs);
		}
		return true;
	}

	std::vector<uint32_t> CompileReferenceWords(const Node& tree)
	{
		std::vector<uint32_t> w;
		ReferenceWords(tree, w);
		w.push_back(OpStop);
		return w;
	}

	void CompiledTree::CopyCode(float* dst) const
	{
		// The chunks to their offsets on the worker pool when there is enough to copy (a
		// 256-primitive tree's program image is about 2.5 MB).
		std::vector<size_t> at(CodeChunks.size());
		size_t off = 0;
		for (size_t i = 0; i < CodeChunks.size(); ++i) { at[i] = off; off += CodeChunks[i].size(); }
		auto copy = [&](int i) { std::memcpy(dst + at[(size_t)i], CodeChunks[(size_t)i].data(), CodeChunks[(size_t)i].size() * sizeof(float)); };
		if (off * sizeof(float) >= ((size_t)1 << 20)) WorkerPool::Get().ParallelFor((int)CodeChunks.size(), copy);
		else for (size_t i = 0; i < CodeChunks.size(); ++i) copy((int)i);
	}

	// What FinishSurfaces needs: the trees (the full tree and, through the octree's cells,
	// every distinct evaluator), the brush records, and where each surface program goes.
	// Dropping it hands the octree's clipped trees to the background thread.
	struct DeferredSurfaces
	{
		NodeRef Root;
		std::shared_ptr<std::vector<Octree::Cell>> Cells;
		std::unordered_map<const Material*, int> Materials;
		std::vector<float> Unused;
		std::unique_ptr<Emitter> Shared;
		std::vector<const Node*> Items;     // the distinct evaluators, then the full tree
		std::vector<int> SurfaceAt;         // each item's surface program: first quad in the image
		std::vector<int> SurfaceQuads;      // and its quads, stop included
		std::vector<int> ChunkFirst;        // first item of each emission chunk (chunks + 1)
		std::vector<int> ChunkBase;         // first quad of each chunk in the image
		~DeferredSurfaces()
		{
			Shared.reset();
			if (Cells)
			{
				auto cells = std::move(Cells);
				WorkerPool::Get().Later([cells]() { cells->clear(); });
			}
		}
	};

	bool FinishSurfaces(CompiledTree& t, float* image, std::string& error)
	{
		std::shared_ptr<DeferredSurfaces> ds = std::move(t.Pending);
		if (!ds) return true;
		const int chunks = (int)ds->ChunkFirst.size() - 1;
		std::atomic<bool> ok{ true };
		WorkerPool::Get().ParallelFor(chunks, [&](int ch)
		{
			std::vector<float> code;
			code.reserve(1 << 12);
			Emitter em(code, ds->Materials, ds->Shared.get());
			float* dst = image ? image : t.CodeChunks[(size_t)ch + 1].data();
			const int base = image ? 0 : ds->ChunkBase[(size_t)ch];
			for (int u = ds->ChunkFirst[(size_t)ch]; u < ds->ChunkFirst[(size_t)ch + 1]; ++u)
			{
				code.clear();
				em.Surface(*ds->Items[(size_t)u]);
				em.Quad(OpStop, 0.0f, 0.0f, 0.0f);
				if (code.size() != (size_t)ds->SurfaceQuads[(size_t)u] * 4)
				{
					ok.store(false);
					continue;
				}
				std::memcpy(dst + (size_t)(ds->SurfaceAt[(size_t)u] - base) * 4, code.data(), code.size() * sizeof(float));
			}
		});
		if (!ok.load())
		{
			error = "a surface program's size differs from its laid-out size";
			return false;
		}
		return true;
	}

	bool CompileTree(const NodeRef& root, CompiledTree& out, std::string& error, OctreeKind kind, const RootHook* on_root,
		bool defer_surfaces)
	{
		const auto t0 = std::chrono::steady_clock::now();
		if (!root)
		{
			error = "the tree has infinite or empty bounds (SDFOctree::Create would return null)";
			return false;
		}
		auto ds = std::make_shared<DeferredSurfaces>();
		ds->Root = root;
		std::vector<const Material*> materialList;
		CollectMaterials(*root, ds->Materials, materialList);
		// Every brush of the full tree (clipped trees share them) gets its records once, up
		// front, and every node of it its surface program's size; the emitters only copy
		// spans of the records.
		ds->Shared.reset(new Emitter(ds->Unused, ds->Materials));
		Emitter& shared = *ds->Shared;
		shared.BuildAllRecords(*root);
		if (defer_surfaces)
		{
			int q, pk;
			shared.SurfaceSize(*root, q, pk);
		}
		// The root cell's program, emitted as the programs below emit node 0's.
		Octree::RootSeen rootSeen;
		if (on_root && *on_root && kind == OctreeKind::Export)
		{
			rootSeen = [&](const Vec3& pivot, float radius, const NodeRef& evaluator)
			{
				RootProgram rp;
				Emitter em(rp.Code, ds->Materials, &shared);
				const int depth = em.Distance(*evaluator);
				em.Quad(OpStop, 0.0f, 0.0f, 0.0f);
				if (depth > kMaxStack) return;   // the compile fails on it below
				OctNode& n = rp.Node;
				n.Pivot[0] = pivot.x; n.Pivot[1] = pivot.y; n.Pivot[2] = pivot.z;
				n.Flags = kNodeTerminus;
				for (int k = 0; k < 8; ++k) n.Child[k] = -1;
				n.DistanceCode = 0;
				n.SurfaceCode = (int32_t)(rp.Code.size() / 4);
				n.StackSize = depth;
				n.ClipRadius = em.NonLipschitz ? -radius : radius;
				(*on_root)(rp);
			};
		}
		const auto ta = std::chrono::steady_clock::now();
		Octree octree;
		if (!(kind == OctreeKind::Meshing ? octree.BuildMeshing(root) : octree.Build(root, 0.25f, true, -1, &rootSeen)))
		{
			error = "the tree has infinite or empty bounds (SDFOctree::Create would return null)";
			return false;
		}
		const auto t1 = std::chrono::steady_clock::now();
		out = CompiledTree();
		out.OctreeSeconds = std::chrono::duration<double>(t1 - ta).count();
		out.Bounds = root->Bounds();
		out.OctreeBounds = octree.Cells[0].Bounds;
		// Each distinct evaluator's two programs are laid out once (cells whose clip left the
		// parent's subtree untouched share its node, RebuildSet), in parallel over chunks of
		// the distinct evaluators, each chunk into its own buffer with its own emitter; the
		// buffers are then laid end to end in chunk order, so the layout does not depend on
		// the threads' timing.  A chunk holds, per evaluator, its distance program and stop,
		// then its surface program and stop; with defer_surfaces the surface program's place
		// is only sized and zero-filled here, and FinishSurfaces emits it.
		struct EmittedPrograms { int Distance, Surface, Stack; bool NonLipschitz; };
		std::vector<const Node*>& distinct = ds->Items;
		std::vector<int> programOf(octree.Cells.size(), -1);
		{
			// Open addressing on the node address, first appearance order.
			size_t cap = 64;
			while (cap < octree.Cells.size() * 2) cap <<= 1;
			std::vector<std::pair<const Node*, int>> index(cap, { nullptr, -1 });
			for (size_t i = 0; i < octree.Cells.size(); ++i)
			{
				const Node* e = octree.Cells[i].Evaluator.get();
				if (!e) continue;
				size_t h = (size_t)(((uint64_t)(uintptr_t)e >> 4) * 0x9E3779B97F4A7C15ull >> 20) & (cap - 1);
				while (index[h].first && index[h].first != e) h = (h + 1) & (cap - 1);
				if (!index[h].first)
				{
					index[h] = { e, (int)distinct.size() };
					distinct.push_back(e);
				}
				programOf[i] = index[h].second;
			}
		}
		// The last item is the whole tree's surface program, for SDFNode::RayMarch / Eval.
		const size_t evaluators = distinct.size();
		distinct.push_back(root.get());
		const size_t items = distinct.size();
		const int chunkCount = (int)std::min<size_t>(items, (size_t)WorkerPool::Get().Workers() * 4 + 4);
		std::vector<std::vector<float>> chunkCode((size_t)chunkCount);
		std::vector<EmittedPrograms> programs(items);
		ds->SurfaceQuads.assign(items, 0);
		// Chunks of about equal cost, a program's cost taken as its tree's leaf count: the
		// largest programs come first in depth-first order (the root's, its children's), and
		// equal item counts left one chunk far longer than the rest.  Where the boundaries
		// fall does not change the image (chunks are laid end to end in item order).
		{
			std::vector<uint64_t> cost(items, 0);
			for (size_t i = 0; i < octree.Cells.size(); ++i)
			{
				const int u = programOf[i];
				if (u >= 0 && cost[(size_t)u] == 0) cost[(size_t)u] = (uint64_t)std::max(1, octree.Cells[i].EvaluatorLeaves);
			}
			cost[evaluators] = (uint64_t)std::max(1, root->LeafCount());
			uint64_t total = 0;
			for (uint64_t c : cost) total += c;
			ds->ChunkFirst.assign((size_t)chunkCount + 1, (int)items);
			ds->ChunkFirst[0] = 0;
			uint64_t sum = 0;
			int ch = 1;
			for (size_t u = 0; u < items && ch < chunkCount; ++u)
			{
				sum += cost[u];
				while (ch < chunkCount && sum * (uint64_t)chunkCount >= total * (uint64_t)ch) ds->ChunkFirst[(size_t)ch++] = (int)u + 1;
			}
		}
		WorkerPool::Get().ParallelFor(chunkCount, [&](int ch)
		{
			std::vector<float>& code = chunkCode[(size_t)ch];
			code.reserve(1 << 14);
			Emitter em(code, ds->Materials, &shared);
			for (int u = ds->ChunkFirst[(size_t)ch]; u < ds->ChunkFirst[(size_t)ch + 1]; ++u)
			{
				const Node& n = *distinct[(size_t)u];
				int d1 = 0;
				bool nonLipschitz = false;
				const int dist = (int)(code.size() / 4);
				if ((size_t)u != evaluators)
				{
					em.NonLipschitz = false;
					d1 = em.Distance(n);
					em.Quad(OpStop, 0.0f, 0.0f, 0.0f);
					nonLipschitz = em.NonLipschitz;
				}
				const int surf = (int)(code.size() / 4);
				int quads, peak;
				if (defer_surfaces)
				{
					em.SurfaceSize(n, quads, peak);
					code.resize(code.size() + (size_t)(quads + 1) * 4, 0.0f);
				}
				else
				{
					peak = em.Surface(n);
					em.Quad(OpStop, 0.0f, 0.0f, 0.0f);
					quads = (int)(code.size() / 4) - surf - 1;
				}
				programs[(size_t)u] = (size_t)u == evaluators ? EmittedPrograms{ surf, surf, peak, false }
					: EmittedPrograms{ dist, surf, d1 > peak ? d1 : peak, nonLipschitz };
				ds->SurfaceQuads[(size_t)u] = quads + 1;
			}
		});
		// One stop record first (the programs of cells without an evaluator), then the
		// chunks in order; they are not copied together here (the upload packs them).
		out.CodeChunks.reserve((size_t)chunkCount + 1);
		out.CodeChunks.push_back({ BitsFloat(OpStop), 0.0f, 0.0f, 0.0f });
		out.CodeFloats = 4;
		const int stopQuad = 0;
		ds->ChunkBase.resize((size_t)chunkCount);
		ds->SurfaceAt.resize(items);
		for (int ch = 0; ch < chunkCount; ++ch)
		{
			const int base = (int)(out.CodeFloats / 4);
			ds->ChunkBase[(size_t)ch] = base;
			for (int u = ds->ChunkFirst[(size_t)ch]; u < ds->ChunkFirst[(size_t)ch + 1]; ++u)
			{
				programs[(size_t)u].Distance += base;
				programs[(size_t)u].Surface += base;
				ds->SurfaceAt[(size_t)u] = programs[(size_t)u].Surface;
			}
			out.CodeFloats += chunkCode[(size_t)ch].size();
			out.CodeChunks.push_back(std::move(chunkCode[(size_t)ch]));
		}
		int maxStack = 0;
		out.Nodes.resize(octree.Cells.size());
		for (size_t i = 0; i < octree.Cells.size(); ++i)
		{
			const Octree::Cell& c = octree.Cells[i];
			OctNode& n = out.Nodes[i];
			n.Pivot[0] = c.Pivot.x; n.Pivot[1] = c.Pivot.y; n.Pivot[2] = c.Pivot.z;
			n.Flags = (c.Terminus ? kNodeTerminus : 0) | (int32_t)(c.NullOctants << 8);
			for (int k = 0; k < 8; ++k) n.Child[k] = c.Children[k];
			if (!c.Evaluator)
			{
				// Only the meshing octree's second stage leaves such cells; descents pass
				// over them.
				n.Flags |= kNodeNoEvaluator;
				n.DistanceCode = n.SurfaceCode = stopQuad;
				n.StackSize = 0;
				n.ClipRadius = c.ClipRadius;
				continue;
			}
			if (kind == OctreeKind::Meshing && c.Terminus) out.LeafBounds.push_back(c.Bounds);
			const EmittedPrograms& e = programs[(size_t)programOf[i]];
			n.DistanceCode = e.Distance;
			n.SurfaceCode = e.Surface;
			n.StackSize = e.Stack;
			n.ClipRadius = e.NonLipschitz ? -c.ClipRadius : c.ClipRadius;
			if (n.StackSize > maxStack) maxStack = n.StackSize;
			out.DistanceQuadsTotal += e.Surface - e.Distance;
		}
		const int full = programs[evaluators].Surface;
		if (programs[evaluators].Stack > maxStack) maxStack = programs[evaluators].Stack;
		out.Header.FullSurfaceCode = full;
		out.Header.Lipschitz = HasNonLipschitzBrush(*root) ? 0 : 1;
		if (maxStack > kMaxStack)
		{
			error = "tree needs a deeper evaluation stack than the kernels hold";
			return false;
		}
		out.Colors.resize(materialList.size() * 4);
		for (size_t m = 0; m < materialList.size(); ++m)
		{
			for (int ch = 0; ch < 3; ++ch)
			{
				// uint8_t(0xFF * c): truncation, as WritePLY(Octree, ...) stores it (export.cpp:309-311).
				const float v = 255.0f * materialList[m]->Rgb[ch];
				out.Colors[m * 4 + ch] = (uint8_t)v;
			}
			out.Colors[m * 4 + 3] = 255;
		}
		out.MaterialRgb.resize(materialList.size() * 4);
		for (size_t m = 0; m < materialList.size(); ++m)
		{
			for (int ch = 0; ch < 3; ++ch) out.MaterialRgb[m * 4 + ch] = materialList[m]->Rgb[ch];
			out.MaterialRgb[m * 4 + 3] = 1.0f;
		}
		out.Header.NodeCount = (int32_t)out.Nodes.size();
		out.Header.CodeQuads = (int32_t)(out.CodeFloats / 4);
		out.Header.MaterialCount = (int32_t)materialList.size();
		out.Header.HasPaint = octree.Cells[0].Evaluator->HasPaint() ? 1 : 0;
		out.Header.MaxStack = maxStack;
		// Releasing thousands of clipped subtrees takes about a millisecond; the caller does
		// not need to wait for it (it touches only the nodes the clips made: the rest are
		// borrowed, and counts are atomic).  They go once the surface programs are emitted.
		ds->Cells = std::make_shared<std::vector<Octree::Cell>>(std::move(octree.Cells));
		if (defer_surfaces) out.Pending = std::move(ds);
		out.BuildSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
		return true;
	}
}
