// Two lattice points per thread in Blackwell's paired FP32 instructions.
//
// sm_100-class GPUs run two independent float32 operations of the same kind on a register
// pair in one instruction.  The distance formulas of tg_sdfmath.hpp are restated here on
// float2 pairs -- point 0 in .x, point 1 in .y -- with every multiply and add in the same
// order as the scalar form, so each lane's result is bit-identical to the scalar
// interpreter's; only the issue count halves.  Square roots, comparisons, min/max and the
// blend term stay scalar per lane (they have no paired forms).
#pragma once

#include <cuda_runtime.h>

#include "../host/tg_sdfmath.hpp"

namespace tg
{
	__device__ __forceinline__ float2 Pair(float s) { return make_float2(s, s); }

	// The paired add and multiply as paired fused multiply-adds that round once each: a * b
	// is fma(a, b, -0) and a + b is fma(a, 1, b), exactly the IEEE product and sum (the
	// exact value of a*b - 0 is a*b, signed zeros included, and a*1 is exact).  The 1 and
	// the -0 are read from memory at run time (PairUnits), so the code generator cannot
	// tell these fmas from general ones and merge a product into the sum that consumes it
	// (with compile-time constants, or as plain paired multiplies and adds, it does, and
	// the results differ from the reference's separately rounded products and sums;
	// tg_debug_pair_check tests every lane).
	static __device__ float g_pair_units[2] = { 1.0f, -0.0f };

	struct PairUnits
	{
		float one, negzero;
	};

	__device__ __forceinline__ PairUnits LoadPairUnits()
	{
		return { *(volatile float*)&g_pair_units[0], *(volatile float*)&g_pair_units[1] };
	}

	__device__ __forceinline__ float2 Add2(float2 a, float2 b, const PairUnits& u)
	{
		float2 r;
		asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
			"mov.b64 pc, {%6, %6};\n\tfma.rn.f32x2 pd, pa, pc, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
			: "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(u.one));
		return r;
	}

	__device__ __forceinline__ float2 Mul2(float2 a, float2 b, const PairUnits& u)
	{
		float2 r;
		asm("{\n\t.reg .b64 pa, pb, pc, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
			"mov.b64 pc, {%6, %6};\n\tfma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;\n\t}"
			: "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(u.negzero));
		return r;
	}

	// a - b = a + (-b) exactly (negation is exact, signed zeros included).
	__device__ __forceinline__ float2 Sub2(float2 a, float2 b, const PairUnits& u) { return Add2(a, make_float2(-b.x, -b.y), u); }
	__device__ __forceinline__ float2 Abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
	__device__ __forceinline__ float2 Sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
	__device__ __forceinline__ float2 TernaryMax2(float2 a, float b) { return make_float2(TernaryMax(a.x, b), TernaryMax(a.y, b)); }

	// Dot(v, v) = (x*x + y*y) + z*z (tg_math.hpp Dot: t.x + t.y + t.z).
	__device__ __forceinline__ float2 Dot3Self2(float2 x, float2 y, float2 z, const PairUnits& u)
	{
		const float2 xx = Mul2(x, x, u), yy = Mul2(y, y, u), zz = Mul2(z, z, u);
		return Add2(Add2(xx, yy, u), zz, u);
	}

	// Length2 of a 2-vector: sqrt(x*x + y*y).
	__device__ __forceinline__ float2 Length22(float2 x, float2 y, const PairUnits& u)
	{
		return Sqrt2(Add2(Mul2(x, x, u), Mul2(y, y, u), u));
	}

	__device__ __forceinline__ float2 SdSphere2(float2 x, float2 y, float2 z, float r, const PairUnits& u)
	{
		return Sub2(Sqrt2(Dot3Self2(x, y, z, u)), Pair(r), u);
	}

	__device__ __forceinline__ float2 SdBox2(float2 x, float2 y, float2 z, float ex, float ey, float ez, const PairUnits& u)
	{
		const float2 ax = Sub2(Abs2(x), Pair(ex), u), ay = Sub2(Abs2(y), Pair(ey), u), az = Sub2(Abs2(z), Pair(ez), u);
		const float2 len = Sqrt2(Dot3Self2(TernaryMax2(ax, 0.0f), TernaryMax2(ay, 0.0f), TernaryMax2(az, 0.0f), u));
		const float2 inner = make_float2(fminf(fmaxf(fmaxf(ax.x, ay.x), az.x), 0.0f), fminf(fmaxf(fmaxf(ax.y, ay.y), az.y), 0.0f));
		return Add2(len, inner, u);
	}

	__device__ __forceinline__ float2 SdTorus2(float2 x, float2 y, float2 z, float major, float minor, const PairUnits& u)
	{
		const float2 ring = Sub2(Length22(x, y, u), Pair(major), u);
		return Sub2(Length22(ring, z, u), Pair(minor), u);
	}

	__device__ __forceinline__ float2 SdCylinder2(float2 x, float2 y, float2 z, float radius, float extent, const PairUnits& u)
	{
		const float2 dx = Sub2(Abs2(Length22(x, y, u)), Pair(radius), u), dy = Sub2(Abs2(z), Pair(extent), u);
		const float2 inner = make_float2(fminf(fmaxf(dx.x, dy.x), 0.0f), fminf(fmaxf(dx.y, dy.y), 0.0f));
		return Add2(inner, Length22(TernaryMax2(dx, 0.0f), TernaryMax2(dy, 0.0f), u), u);
	}

	// SdPlane: Dot(p, n) = (x*nx + y*ny) + z*nz.
	__device__ __forceinline__ float2 SdPlane2(float2 x, float2 y, float2 z, float nx, float ny, float nz, const PairUnits& u)
	{
		const float2 a = Mul2(x, Pair(nx), u), b = Mul2(y, Pair(ny), u), c = Mul2(z, Pair(nz), u);
		return Add2(Add2(a, b, u), c, u);
	}

	// One row m of the affine transform (M * vec4(p, 1)): (m0*x + m1*y) + (m2*z + m3).
	__device__ __forceinline__ float2 AffineRow2(float4 m, float2 x, float2 y, float2 z, const PairUnits& u)
	{
		const float2 a = Mul2(Pair(m.x), x, u), b = Mul2(Pair(m.y), y, u), c = Mul2(Pair(m.z), z, u);
		return Add2(Add2(a, b, u), Add2(c, Pair(m.w), u), u);
	}

	__device__ __forceinline__ float2 BrushDistance2(uint32_t op, const float (&prm)[3], float2 x, float2 y, float2 z, const PairUnits& u)
	{
		switch (op)
		{
		case OpSphere: return SdSphere2(x, y, z, prm[0], u);
		case OpBox: return SdBox2(x, y, z, prm[0], prm[1], prm[2], u);
		case OpTorus: return SdTorus2(x, y, z, prm[0], prm[1], u);
		case OpCylinder: return SdCylinder2(x, y, z, prm[0], prm[1], u);
		case OpPlane: return SdPlane2(x, y, z, prm[0], prm[1], prm[2], u);
		default:
			return make_float2(BrushDistance(op, prm, Vec3(x.x, y.x, z.x)), BrushDistance(op, prm, Vec3(x.y, y.y, z.y)));
		}
	}

	__device__ __forceinline__ float2 SetDistance2(uint32_t op, float2 l, float2 r, float k)
	{
		if (op == OpUnion) return make_float2(fminf(l.x, r.x), fminf(l.y, r.y));
		return make_float2(SetDistance(op, l.x, r.x, k), SetDistance(op, l.y, r.y, k));
	}

	// RunDistance (tg_device.cuh) for NP pairs of points at once (2 NP points): pair j is
	// (px[j].x, py[j].x, pz[j].x) and (px[j].y, py[j].y, pz[j].y).  `spill` is this
	// thread's column of the operand stack in shared memory: entry (depth, pair j) at
	// spill[(depth * NP + j) * stride] (a float2).  `load(q)` returns record quad q of the
	// program (from global or shared memory).
	template<int NP, typename Load>
	__device__ __forceinline__ void RunDistancePairs(Load load, int pc, const float2 (&px)[NP], const float2 (&py)[NP],
		const float2 (&pz)[NP], float2 (&out)[NP], float2* spill, int stride)
	{
		const PairUnits u = LoadPairUnits();
		float2 acc[NP];
#pragma unroll
		for (int j = 0; j < NP; ++j) acc[j] = make_float2(0.0f, 0.0f);
		int depth = 0;
		for (int guard = 0; guard < (1 << 24); ++guard)
		{
			const float4 h = load(pc++);
			const uint32_t head = __float_as_uint(h.x);
			const uint32_t op = head & 0xFFu;
			if (op >= OpSphere && op <= OpPlane)
			{
				const bool thenSet = (head & RecThenSet) != 0;
				float2 left[NP];
#pragma unroll
				for (int j = 0; j < NP; ++j) left[j] = acc[j];
				if (!thenSet)
				{
					if (depth > 0)
					{
#pragma unroll
						for (int j = 0; j < NP; ++j) spill[((depth - 1) * NP + j) * stride] = acc[j];
					}
					++depth;
				}
				float2 qx[NP], qy[NP], qz[NP];
#pragma unroll
				for (int j = 0; j < NP; ++j) { qx[j] = px[j]; qy[j] = py[j]; qz[j] = pz[j]; }
				if (head & RecMatrix)
				{
					const float4 X = load(pc), Y = load(pc + 1), Z = load(pc + 2);
					pc += 3;
#pragma unroll
					for (int j = 0; j < NP; ++j)
					{
						qx[j] = AffineRow2(X, px[j], py[j], pz[j], u);
						qy[j] = AffineRow2(Y, px[j], py[j], pz[j], u);
						qz[j] = AffineRow2(Z, px[j], py[j], pz[j], u);
					}
				}
				else if (head & RecOffset)
				{
					const float4 O = load(pc++);
#pragma unroll
					for (int j = 0; j < NP; ++j)
					{
						qx[j] = Add2(px[j], Pair(O.x), u);
						qy[j] = Add2(py[j], Pair(O.y), u);
						qz[j] = Add2(pz[j], Pair(O.z), u);
					}
				}
				const float prm[3] = { h.y, h.z, h.w };
#pragma unroll
				for (int j = 0; j < NP; ++j) acc[j] = BrushDistance2(op, prm, qx[j], qy[j], qz[j], u);
				if (head & RecScale)
				{
					const float4 S = load(pc++);
#pragma unroll
					for (int j = 0; j < NP; ++j) acc[j] = Mul2(acc[j], Pair(S.x), u);
				}
				if (thenSet)
				{
					const float4 T = load(pc++);
					const uint32_t setOp = __float_as_uint(T.x) & 0xFFu;
#pragma unroll
					for (int j = 0; j < NP; ++j) acc[j] = SetDistance2(setOp, left[j], acc[j], T.y);
				}
			}
			else if (op >= OpUnion && op <= OpBlendDiff)
			{
				--depth;
#pragma unroll
				for (int j = 0; j < NP; ++j) acc[j] = SetDistance2(op, spill[((depth - 1) * NP + j) * stride], acc[j], h.y);
			}
			else if (op == OpFlate)
			{
#pragma unroll
				for (int j = 0; j < NP; ++j) acc[j] = Sub2(acc[j], Pair(h.y), u);
			}
			else
			{
				break;   // OpStop
			}
		}
#pragma unroll
		for (int j = 0; j < NP; ++j) out[j] = acc[j];
	}

	// RunDistance<K> through the paired instructions, for even K: point k is lane k % 2 of
	// pair k / 2.  `spill` as RunDistance's (K floats per stack entry and thread).
	template<int K, typename Load>
	__device__ __forceinline__ void RunDistancePaired(Load load, int pc, const float (&px)[K], const float (&py)[K], const float (&pz)[K],
		float (&out)[K], float* spill, int stride)
	{
		static_assert(K % 2 == 0, "paired evaluation takes an even number of points");
		constexpr int NP = K / 2;
		float2 x[NP], y[NP], z[NP], r[NP];
#pragma unroll
		for (int j = 0; j < NP; ++j)
		{
			x[j] = make_float2(px[2 * j], px[2 * j + 1]);
			y[j] = make_float2(py[2 * j], py[2 * j + 1]);
			z[j] = make_float2(pz[2 * j], pz[2 * j + 1]);
		}
		RunDistancePairs<NP>(load, pc, x, y, z, r, reinterpret_cast<float2*>(spill), stride);
#pragma unroll
		for (int j = 0; j < NP; ++j) { out[2 * j] = r[j].x; out[2 * j + 1] = r[j].y; }
	}

	// Cross(a, b) of tg_math.hpp for a uniform a and a pair b:
	// { a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y }.
	__device__ __forceinline__ void CrossPair(float ax, float ay, float az, float2 bx, float2 by, float2 bz,
		float2& cx, float2& cy, float2& cz, const PairUnits& u)
	{
		cx = Sub2(Mul2(Pair(ay), bz, u), Mul2(by, Pair(az), u), u);
		cy = Sub2(Mul2(Pair(az), bx, u), Mul2(bz, Pair(ax), u), u);
		cz = Sub2(Mul2(Pair(ax), by, u), Mul2(bx, Pair(ay), u), u);
	}

	// SDFNode::Eval through a surface program (RunSurfaceBatch in tg_device.cuh without the
	// material walk) for one pair of points: every brush rotates the point by its inverse
	// quaternion, q * v = v + ((cross(q.xyz, v) * w) + cross(q.xyz, cross(q.xyz, v))) * 2,
	// after subtracting its translation, divides by its scale (skipped at scale 1: x / 1 is
	// x), and multiplies the brush distance by the scale.  `spill`: entry `depth` at
	// spill[depth * stride] (a float2).
	template<typename Load>
	__device__ __forceinline__ float2 RunSurfacePair(Load load, int pc, float2 px, float2 py, float2 pz, float2* spill, int stride)
	{
		const PairUnits u = LoadPairUnits();
		float2 acc = make_float2(0.0f, 0.0f);
		int depth = 0;
		for (int guard = 0; guard < (1 << 24); ++guard)
		{
			const float4 h = load(pc++);
			const uint32_t head = __float_as_uint(h.x);
			const uint32_t op = head & 0xFFu;
			if (op >= OpSphere && op <= OpPlane)
			{
				const bool thenSet = (head & RecThenSet) != 0;
				const float2 left = acc;
				if (!thenSet)
				{
					if (depth > 0) spill[(depth - 1) * stride] = acc;
					++depth;
				}
				const float4 Q = load(pc);
				const float4 T = load(pc + 1);
				pc += 3;
				const float2 vx = Sub2(px, Pair(T.x), u), vy = Sub2(py, Pair(T.y), u), vz = Sub2(pz, Pair(T.z), u);
				// The quad holds the inverse quaternion as (w, x, y, z).
				float2 ux, uy, uz, wx, wy, wz;
				CrossPair(Q.y, Q.z, Q.w, vx, vy, vz, ux, uy, uz, u);
				CrossPair(Q.y, Q.z, Q.w, ux, uy, uz, wx, wy, wz, u);
				float2 lx = Add2(vx, Mul2(Add2(Mul2(ux, Pair(Q.x), u), wx, u), Pair(2.0f), u), u);
				float2 ly = Add2(vy, Mul2(Add2(Mul2(uy, Pair(Q.x), u), wy, u), Pair(2.0f), u), u);
				float2 lz = Add2(vz, Mul2(Add2(Mul2(uz, Pair(Q.x), u), wz, u), Pair(2.0f), u), u);
				const bool scaled = T.w != 1.0f;
				if (scaled)
				{
					lx = make_float2(lx.x / T.w, lx.y / T.w);
					ly = make_float2(ly.x / T.w, ly.y / T.w);
					lz = make_float2(lz.x / T.w, lz.y / T.w);
				}
				const float prm[3] = { h.y, h.z, h.w };
				float2 d = BrushDistance2(op, prm, lx, ly, lz, u);
				if (scaled) d = Mul2(d, Pair(T.w), u);
				acc = d;
				if (thenSet)
				{
					const float4 S = load(pc++);
					acc = SetDistance2(__float_as_uint(S.x) & 0xFFu, left, acc, S.y);
				}
			}
			else if (op >= OpUnion && op <= OpBlendDiff)
			{
				--depth;
				acc = SetDistance2(op, spill[(depth - 1) * stride], acc, h.y);
			}
			else if (op == OpFlate)
			{
				acc = Sub2(acc, Pair(h.y), u);
			}
			else if (op == OpMaskBegin)
			{
				pc += (int)__float_as_uint(h.y);
			}
			else if (op == OpStencilEnd)
			{
				--depth;
				acc = spill[(depth - 1) * stride];
			}
			else
			{
				break;   // OpStop
			}
		}
		return acc;
	}
}
