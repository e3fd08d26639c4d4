// Device-side evaluation of compiled trees (record format: tg_layout.hpp).
//
// Every kernel translation unit that includes this header is compiled with -fmad=false:
// the reference's x86-64 Release build never fuses a multiply and an add, and bit-exact
// distances need the same roundings.  Division and square root are IEEE (no fast math).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../host/tg_layout.hpp"
#include "../host/tg_sdfmath.hpp"

namespace tg
{
	// World coordinate of lattice index i: x0 + float(i) * step, the rounding the export
	// grid uses (surface_nets.cpp get_world_point_of / get_voxel_corner_world_positions).
	__device__ __forceinline__ float LatticeCoord(float origin, int i, float step)
	{
		return origin + static_cast<float>(i) * step;
	}

	// SDFOctree::Descend(Point, Exact = true) (sdf_evaluator.cpp:1801-1835): follow the
	// pivot octant while a child exists; a missing child means this cell's own evaluator.
	__device__ __forceinline__ int DescendOctree(const OctNode* __restrict__ nodes, float x, float y, float z)
	{
		int at = 0;
		for (int guard = 0; guard < 64; ++guard)
		{
			const float4 a = __ldg(reinterpret_cast<const float4*>(nodes + at));
			if (__float_as_int(a.w) & kNodeTerminus) break;
			const int octant = (x > a.x ? 1 : 0) | (y > a.y ? 2 : 0) | (z > a.z ? 4 : 0);
			const int child = __ldg(&nodes[at].Child[octant]);
			if (child < 0) break;
			at = child;
		}
		return at;
	}

	// DescendOctree continued from cell `at` (an ancestor of the point's cell).
	__device__ __forceinline__ int DescendOctreeFrom(const OctNode* __restrict__ nodes, int at, float x, float y, float z)
	{
		for (int guard = 0; guard < 64; ++guard)
		{
			const float4 a = __ldg(reinterpret_cast<const float4*>(nodes + at));
			if (__float_as_int(a.w) & kNodeTerminus) break;
			const int octant = (x > a.x ? 1 : 0) | (y > a.y ? 2 : 0) | (z > a.z ? 4 : 0);
			const int child = __ldg(&nodes[at].Child[octant]);
			if (child < 0) break;
			at = child;
		}
		return at;
	}

	// The descent of a whole box of points [x0, x1] x [y0, y1] x [z0, z1] as far as they all
	// take the same octant: returns the cell reached, and `shared` = every point of the box
	// descends to exactly that cell (DescendOctree's `p > pivot` rule holds for the whole box
	// when its lower corner is above the pivot, and fails for it when its upper corner is not).
	__device__ __forceinline__ int DescendBox(const OctNode* __restrict__ nodes, float x0, float x1, float y0, float y1, float z0,
		float z1, bool& shared)
	{
		int at = 0;
		shared = false;
		for (int guard = 0; guard < 64; ++guard)
		{
			const float4 a = __ldg(reinterpret_cast<const float4*>(nodes + at));
			if (__float_as_int(a.w) & kNodeTerminus) { shared = true; break; }
			const bool hx = x0 > a.x, lx = !(x1 > a.x);
			const bool hy = y0 > a.y, ly = !(y1 > a.y);
			const bool hz = z0 > a.z, lz = !(z1 > a.z);
			if (!((hx || lx) && (hy || ly) && (hz || lz))) break;
			const int octant = (hx ? 1 : 0) | (hy ? 2 : 0) | (hz ? 4 : 0);
			const int child = __ldg(&nodes[at].Child[octant]);
			if (child < 0) { shared = true; break; }
			at = child;
		}
		return at;
	}

	__device__ __forceinline__ float4 LoadQuad(const float4* __restrict__ code, int q)
	{
		return __ldg(code + q);
	}

	// Runs a distance program for K points at once (one record stream, K accumulators).
	// `spill` is this thread's column of the operand stack in shared memory: entry
	// (depth, lane) lives at spill[(depth * K + lane) * stride].
	// FuseSet = false ignores RecThenSet (the set record is then taken as its own step, with
	// the same result) for kernels whose register budget cannot hold the fused step.
	template<int K, bool FuseSet = true>
	__device__ __forceinline__ void RunDistance(const float4* __restrict__ code, int pc,
		const float (&px)[K], const float (&py)[K], const float (&pz)[K], float (&out)[K],
		float* spill, int stride)
	{
		float acc[K];
#pragma unroll
		for (int k = 0; k < K; ++k) acc[k] = 0.0f;
		int depth = 0;
		for (int guard = 0; guard < (1 << 24); ++guard)
		{
			const float4 h = LoadQuad(code, pc++);
			const uint32_t head = __float_as_uint(h.x);
			const uint32_t op = head & 0xFFu;
			if (op >= OpSphere && op <= OpPlane)
			{
				// RecThenSet: the set operator after this brush takes the current accumulator as
				// its left operand, so nothing is pushed (same operations, same order).
				const bool thenSet = FuseSet && (head & RecThenSet) != 0;
				float left[K];
#pragma unroll
				for (int k = 0; k < K; ++k) left[k] = acc[k];
				if (!thenSet)
				{
					if (depth > 0)
					{
#pragma unroll
						for (int k = 0; k < K; ++k) spill[((depth - 1) * K + k) * stride] = acc[k];
					}
					++depth;
				}
				float qx[K], qy[K], qz[K];
				if (head & RecMatrix)
				{
					const float4 X = LoadQuad(code, pc), Y = LoadQuad(code, pc + 1), Z = LoadQuad(code, pc + 2);
					pc += 3;
#pragma unroll
					for (int k = 0; k < K; ++k)
					{
						// (M * vec4(p, 1)).xyz = (m0*x + m1*y) + (m2*z + m3)
						qx[k] = (X.x * px[k] + X.y * py[k]) + (X.z * pz[k] + X.w);
						qy[k] = (Y.x * px[k] + Y.y * py[k]) + (Y.z * pz[k] + Y.w);
						qz[k] = (Z.x * px[k] + Z.y * py[k]) + (Z.z * pz[k] + Z.w);
					}
				}
				else if (head & RecOffset)
				{
					const float4 O = LoadQuad(code, pc++);
#pragma unroll
					for (int k = 0; k < K; ++k) { qx[k] = px[k] + O.x; qy[k] = py[k] + O.y; qz[k] = pz[k] + O.z; }
				}
				else
				{
#pragma unroll
					for (int k = 0; k < K; ++k) { qx[k] = px[k]; qy[k] = py[k]; qz[k] = pz[k]; }
				}
				const float prm[3] = { h.y, h.z, h.w };
				switch (op)
				{
				case OpSphere:
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = SdSphere(Vec3(qx[k], qy[k], qz[k]), prm[0]);
					break;
				case OpBox:
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = SdBox(Vec3(qx[k], qy[k], qz[k]), Vec3(prm[0], prm[1], prm[2]));
					break;
				case OpTorus:
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = SdTorus(Vec3(qx[k], qy[k], qz[k]), prm[0], prm[1]);
					break;
				case OpCylinder:
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = SdCylinder(Vec3(qx[k], qy[k], qz[k]), prm[0], prm[1]);
					break;
				default:
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = BrushDistance(op, prm, Vec3(qx[k], qy[k], qz[k]));
					break;
				}
				if (head & RecScale)
				{
					const float4 S = LoadQuad(code, pc++);
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = acc[k] * S.x;
				}
				if (thenSet)
				{
					const float4 T = LoadQuad(code, pc++);
					const uint32_t setOp = __float_as_uint(T.x) & 0xFFu;
#pragma unroll
					for (int k = 0; k < K; ++k) acc[k] = SetDistance(setOp, left[k], acc[k], T.y);
				}
			}
			else if (op >= OpUnion && op <= OpBlendDiff)
			{
				--depth;
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					const float l = spill[((depth - 1) * K + k) * stride];
					acc[k] = SetDistance(op, l, acc[k], h.y);
				}
			}
			else if (op == OpFlate)
			{
#pragma unroll
				for (int k = 0; k < K; ++k) acc[k] = acc[k] - h.y;
			}
			else
			{
				break;   // OpStop
			}
		}
#pragma unroll
		for (int k = 0; k < K; ++k) out[k] = acc[k];
	}

	// Surface program: SDFNode::Eval (and, with `material`, GetMaterial) at one point.
	// Returns the distance; *material receives the material index (-1: default white).
	__device__ __forceinline__ float RunSurface(const float4* __restrict__ code, int pc, Vec3 p, bool material, int* material_out)
	{
		float dst[kMaxStack];
		int mat[kMaxStack];
		int depth = 0;
		for (int guard = 0; guard < (1 << 24); ++guard)
		{
			const float4 h = LoadQuad(code, pc++);
			const uint32_t head = __float_as_uint(h.x);
			const uint32_t op = head & 0xFFu;
			if (op >= OpSphere && op <= OpPlane)
			{
				const float4 Q = LoadQuad(code, pc);
				const float4 T = LoadQuad(code, pc + 1);
				const float4 M = LoadQuad(code, pc + 2);
				pc += 3;
				// BrushFn(ApplyInv(p)) * s, ApplyInv(p) = rotate(inverse(q), p - t) / s.  An
				// unscaled brush (s = 1, the common case) skips the divide and the multiply:
				// x / 1 and x * 1 are x exactly.
				const Quat qi{ Q.x, Q.y, Q.z, Q.w };
				Vec3 local = Rotate(qi, p - Vec3(T.x, T.y, T.z));
				if (T.w != 1.0f) local = local / T.w;
				const float prm[3] = { h.y, h.z, h.w };
				float d = BrushDistance(op, prm, local);
				if (T.w != 1.0f) d = d * T.w;
				dst[depth] = d;
				mat[depth] = __float_as_int(M.x);
				++depth;
			}
			else if (op >= OpUnion && op <= OpBlendDiff)
			{
				--depth;
				const float r = dst[depth], l = dst[depth - 1];
				const float d = SetDistance(op, l, r, h.y);
				if (material)
				{
					// SetNode::GetMaterial (sdf_evaluator.cpp:957-1012).
					int m;
					if (op == OpDiff || op == OpBlendDiff) m = mat[depth - 1];
					else
					{
						const bool blend = (op == OpBlendUnion || op == OpBlendInter);
						const bool takeLeft = blend ? (fabsf(l - d) <= fabsf(r - d)) : (d == l);
						if (op == OpUnion || op == OpBlendUnion) m = takeLeft ? mat[depth - 1] : mat[depth];
						else
						{
							const bool lv = (head & RecLhsPaint) != 0, rv = (head & RecRhsPaint) != 0;
							if (lv && rv) m = takeLeft ? mat[depth - 1] : mat[depth];
							else m = lv ? mat[depth - 1] : mat[depth];
						}
					}
					mat[depth - 1] = m;
				}
				dst[depth - 1] = d;
			}
			else if (op == OpFlate)
			{
				dst[depth - 1] = dst[depth - 1] - h.y;
			}
			else if (op == OpMaskBegin)
			{
				if (!material) pc += (int)__float_as_uint(h.y);
			}
			else if (op == OpStencilEnd)
			{
				// StencilMaskNode::GetMaterial (sdf_evaluator.cpp:666-679).
				--depth;
				const bool interior = dst[depth] < 0.0f;
				const bool negative = (head & RecNegative) != 0;
				if (interior == negative) mat[depth - 1] = (int)__float_as_uint(h.y);
			}
			else
			{
				break;   // OpStop
			}
		}
		if (material_out) *material_out = mat[0];
		return dst[0];
	}

	// Surface program at K points in one pass over the records (SDFNode::Eval per point);
	// lane `mat_lane` (or none, when negative) also follows GetMaterial and its result goes
	// to *material_out.  Operands below the top of the stack spill to shared memory:
	// distance (depth, lane) at spill[(depth * (K + 1) + lane) * stride] and the material
	// lane's material index at spill[(depth * (K + 1) + K) * stride].
	template<int K, bool FuseSet = true>
	__device__ __forceinline__ void RunSurfaceBatch(const float4* __restrict__ code, int pc,
		const float (&px)[K], const float (&py)[K], const float (&pz)[K], float (&out)[K],
		int mat_lane, int* material_out, float* spill, int stride)
	{
		float acc[K];
#pragma unroll
		for (int k = 0; k < K; ++k) acc[k] = 0.0f;
		int macc = -1;
		int depth = 0;
		const bool withMaterial = mat_lane >= 0;
		auto slot = [&](int d, int lane) -> float& { return spill[(d * (K + 1) + lane) * stride]; };
		for (int guard = 0; guard < (1 << 24); ++guard)
		{
			const float4 h = LoadQuad(code, pc++);
			const uint32_t head = __float_as_uint(h.x);
			const uint32_t op = head & 0xFFu;
			// SetNode::Eval and SetNode::GetMaterial (sdf_evaluator.cpp:774-780, 957-1012) on the
			// left operands l[] (material ml) and the accumulator (the right operands).
			auto applySet = [&](uint32_t setHead, float k0, const float (&l)[K], int ml)
			{
				const uint32_t setOp = setHead & 0xFFu;
				float lm = 0.0f, rm = 0.0f, dm = 0.0f;
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					const float d = SetDistance(setOp, l[k], acc[k], k0);
					if (k == mat_lane) { lm = l[k]; rm = acc[k]; dm = d; }
					acc[k] = d;
				}
				if (withMaterial)
				{
					const int mr = macc;
					if (setOp == OpDiff || setOp == OpBlendDiff) macc = ml;
					else
					{
						const bool blend = (setOp == OpBlendUnion || setOp == OpBlendInter);
						const bool takeLeft = blend ? (fabsf(lm - dm) <= fabsf(rm - dm)) : (dm == lm);
						if (setOp == OpUnion || setOp == OpBlendUnion) macc = takeLeft ? ml : mr;
						else
						{
							const bool lv = (setHead & RecLhsPaint) != 0, rv = (setHead & RecRhsPaint) != 0;
							if (lv && rv) macc = takeLeft ? ml : mr;
							else macc = lv ? ml : mr;
						}
					}
				}
			};
			if (op >= OpSphere && op <= OpPlane)
			{
				// RecThenSet: the set operator after this brush takes the current accumulator
				// (and material) as its left operand, so nothing is pushed.
				const bool thenSet = FuseSet && (head & RecThenSet) != 0;
				float left[K];
#pragma unroll
				for (int k = 0; k < K; ++k) left[k] = acc[k];
				const int leftMaterial = macc;
				if (!thenSet)
				{
					if (depth > 0)
					{
#pragma unroll
						for (int k = 0; k < K; ++k) slot(depth - 1, k) = acc[k];
						slot(depth - 1, K) = __int_as_float(macc);
					}
					++depth;
				}
				const float4 Q = LoadQuad(code, pc);
				const float4 T = LoadQuad(code, pc + 1);
				const float4 M = LoadQuad(code, pc + 2);
				pc += 3;
				const Quat qi{ Q.x, Q.y, Q.z, Q.w };
				const Vec3 t(T.x, T.y, T.z);
				const float prm[3] = { h.y, h.z, h.w };
				const bool scaled = T.w != 1.0f;    // x / 1 and x * 1 are x exactly
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					// BrushFn(ApplyInv(p)) * s with ApplyInv(p) = rotate(inverse(q), p - t) / s
					Vec3 local = Rotate(qi, Vec3(px[k], py[k], pz[k]) - t);
					if (scaled) local = local / T.w;
					float d = BrushDistance(op, prm, local);
					if (scaled) d = d * T.w;
					acc[k] = d;
				}
				macc = __float_as_int(M.x);
				if (thenSet)
				{
					const float4 S = LoadQuad(code, pc++);
					applySet(__float_as_uint(S.x), S.y, left, leftMaterial);
				}
			}
			else if (op >= OpUnion && op <= OpBlendDiff)
			{
				--depth;
				float l[K];
#pragma unroll
				for (int k = 0; k < K; ++k) l[k] = slot(depth - 1, k);
				applySet(head, h.y, l, withMaterial ? __float_as_int(slot(depth - 1, K)) : -1);
			}
			else if (op == OpFlate)
			{
#pragma unroll
				for (int k = 0; k < K; ++k) acc[k] = acc[k] - h.y;
			}
			else if (op == OpMaskBegin)
			{
				if (!withMaterial) pc += (int)__float_as_uint(h.y);
			}
			else if (op == OpStencilEnd)
			{
				// StencilMaskNode::GetMaterial (sdf_evaluator.cpp:666-679): the mask's value is
				// on top, the child's below it.
				--depth;
				float maskValue = 0.0f;
#pragma unroll
				for (int k = 0; k < K; ++k)
				{
					if (k == mat_lane) maskValue = acc[k];
					acc[k] = slot(depth - 1, k);
				}
				const int childMat = __float_as_int(slot(depth - 1, K));
				const bool interior = maskValue < 0.0f;
				const bool negative = (head & RecNegative) != 0;
				macc = (interior == negative) ? (int)__float_as_uint(h.y) : childMat;
			}
			else
			{
				break;   // OpStop
			}
		}
#pragma unroll
		for (int k = 0; k < K; ++k) out[k] = acc[k];
		if (material_out) *material_out = macc;
	}

	// Gradient (and, optionally, material) at p with one batched pass: lanes 0..3 are the
	// tetrahedral points, lane 4 is p itself (SDFNode::Gradient, sdf_evaluator.cpp:298-333).
	__device__ __forceinline__ Vec3 SurfaceGradientBatch(const float4* __restrict__ code, int pc, Vec3 p, bool material,
		int* material_out, float* spill, int stride)
	{
		const float h = 0.0001f;
		const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
		const Vec3 q0 = p + xyy, q1 = p + yyx, q2 = p + yxy, q3 = p + xxx;
		const float px[5] = { q0.x, q1.x, q2.x, q3.x, p.x };
		const float py[5] = { q0.y, q1.y, q2.y, q3.y, p.y };
		const float pz[5] = { q0.z, q1.z, q2.z, q3.z, p.z };
		float e[5];
		RunSurfaceBatch<5>(code, pc, px, py, pz, e, material ? 4 : -1, material_out, spill, stride);
		Vec3 g = xyy * e[0];
		g = g + yyx * e[1];
		g = g + yxy * e[2];
		g = g + xxx * e[3];
		const float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
		if (ls == 0.0f)
		{
			const float d = e[4];
			return Normalize(Vec3(e[0] - d, e[2] - d, e[1] - d));
		}
		return g / sqrtf(ls);
	}

	// SDFNode::Gradient (sdf_evaluator.cpp:298-333) on a surface program.
	__device__ __forceinline__ Vec3 SurfaceGradient(const float4* __restrict__ code, int pc, Vec3 p)
	{
		const float h = 0.0001f;
		const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
		const float e0 = RunSurface(code, pc, p + xyy, false, nullptr);
		const float e1 = RunSurface(code, pc, p + yyx, false, nullptr);
		const float e2 = RunSurface(code, pc, p + yxy, false, nullptr);
		const float e3 = RunSurface(code, pc, p + xxx, false, nullptr);
		Vec3 g = xyy * e0;
		g = g + yyx * e1;
		g = g + yxy * e2;
		g = g + xxx * e3;
		const float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
		if (ls == 0.0f)
		{
			const float d = RunSurface(code, pc, p, false, nullptr);
			return Normalize(Vec3(e0 - d, e2 - d, e1 - d));
		}
		return g / sqrtf(ls);
	}
}
