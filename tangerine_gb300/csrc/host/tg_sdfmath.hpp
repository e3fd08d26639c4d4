// Signed-distance formulas of Tangerine's primitives and set operators
// (tangerine/sdf_evaluator.cpp:165-295), shared verbatim by the host (clip decisions,
// point queries) and the CUDA kernels, so both sides compute the same float32 results.
//
// Arithmetic types follow the reference: where it mixes a float expression with a double
// literal (Ellipsoid's K0 - 1.0, the blend operators' * 0.25, Cone's Height * -.5) the
// expression is evaluated in double and rounded once to float, as C++ does there.
#pragma once

#include "tg_math.hpp"

namespace tg
{
	// Interpreter op codes (OpcodeT, tangerine/sdf_evaluator.h:83-107).
	enum Opcode : uint32_t
	{
		OpStop = 0,
		OpSphere, OpEllipsoid, OpBox, OpTorus, OpCylinder, OpCone, OpConinder, OpPlane,
		OpUnion, OpInter, OpDiff, OpBlendUnion, OpBlendInter, OpBlendDiff, OpFlate,
		OpOffset, OpMatrix, OpScaleField,
	};

	TG_HD int BrushParamCount(uint32_t op)
	{
		return op == OpSphere ? 1 : (op == OpTorus || op == OpCylinder || op == OpCone) ? 2 : 3;
	}

	TG_HD bool IsBrushOp(uint32_t op) { return op >= OpSphere && op <= OpPlane; }
	TG_HD bool IsSetOp(uint32_t op) { return op >= OpUnion && op <= OpBlendDiff; }
	TG_HD bool IsBlendOp(uint32_t op) { return op >= OpBlendUnion && op <= OpBlendDiff; }

	struct Vec2f { float x, y; };
	TG_HD float Dot2(Vec2f a, Vec2f b) { return a.x * b.x + a.y * b.y; }
	TG_HD float Length2(Vec2f a) { return sqrtf(Dot2(a, a)); }
	TG_HD float Sign(float x) { return (float)((0.0f < x) - (x < 0.0f)); }
	TG_HD float TernaryClamp(float x, float lo, float hi) { return TernaryMin(TernaryMax(x, lo), hi); }

	TG_HD float SdSphere(Vec3 p, float r) { return Length(p) - r; }

	TG_HD float SdEllipsoid(Vec3 p, Vec3 r)
	{
		const float k0 = Length(Vec3(p.x / r.x, p.y / r.y, p.z / r.z));
		const Vec3 rr = r * r;
		const float k1 = Length(Vec3(p.x / rr.x, p.y / rr.y, p.z / rr.z));
		return (float)((double)k0 * ((double)k0 - 1.0) / (double)k1);
	}

	TG_HD float SdBox(Vec3 p, Vec3 e)
	{
		const Vec3 a = Abs(p) - e;
		return Length(TernaryMax(a, Vec3(0.0f))) + fminf(fmaxf(fmaxf(a.x, a.y), a.z), 0.0f);
	}

	TG_HD float SdTorus(Vec3 p, float major, float minor)
	{
		return Length2(Vec2f{ Length2(Vec2f{ p.x, p.y }) - major, p.z }) - minor;
	}

	TG_HD float SdCylinder(Vec3 p, float radius, float extent)
	{
		const Vec2f d{ fabsf(Length2(Vec2f{ p.x, p.y })) - radius, fabsf(p.z) - extent };
		return fminf(fmaxf(d.x, d.y), 0.0f) + Length2(Vec2f{ TernaryMax(d.x, 0.0f), TernaryMax(d.y, 0.0f) });
	}

	TG_HD float SdPlane(Vec3 p, Vec3 n) { return Dot(p, n); }

	TG_HD float SdCone(Vec3 p, float tangent, float height)
	{
		const Vec2f q{ height * tangent, height * -1.0f };
		const Vec2f w{ Length2(Vec2f{ p.x, p.y }), (float)((double)height * -0.5 + (double)p.z) };
		const float ca = TernaryClamp(Dot2(w, q) / Dot2(q, q), 0.0f, 1.0f);
		const Vec2f a{ w.x - q.x * ca, w.y - q.y * ca };
		const float cb = TernaryClamp(w.x / q.x, 0.0f, 1.0f);
		const Vec2f b{ w.x - q.x * cb, w.y - q.y * 1.0f };
		const float k = Sign(q.y);
		const float d = fminf(Dot2(a, a), Dot2(b, b));
		const float s = fmaxf(k * (w.x * q.y - w.y * q.x), k * (w.y - q.y));
		return sqrtf(d) * Sign(s);
	}

	TG_HD float SdConinder(Vec3 p, float rl, float rh, float h)
	{
		const Vec2f q{ Length2(Vec2f{ p.x, p.y }), p.z };
		const Vec2f k1{ rh, h };
		const Vec2f k2{ rh - rl, (float)(2.0 * (double)h) };
		const Vec2f ca{ q.x - fminf(q.x, (q.y < 0.0f) ? rl : rh), fabsf(q.y) - h };
		const float c = TernaryClamp(Dot2(Vec2f{ k1.x - q.x, k1.y - q.y }, k2) / Dot2(k2, k2), 0.0f, 1.0f);
		const Vec2f cb{ (q.x - k1.x) + k2.x * c, (q.y - k1.y) + k2.y * c };
		const float s = (cb.x < 0.0f && ca.y < 0.0f) ? -1.0f : 1.0f;
		return s * sqrtf(fminf(Dot2(ca, ca), Dot2(cb, cb)));
	}

	TG_HD float BrushDistance(uint32_t op, const float* prm, Vec3 p)
	{
		switch (op)
		{
		case OpSphere: return SdSphere(p, prm[0]);
		case OpEllipsoid: return SdEllipsoid(p, Vec3(prm[0], prm[1], prm[2]));
		case OpBox: return SdBox(p, Vec3(prm[0], prm[1], prm[2]));
		case OpTorus: return SdTorus(p, prm[0], prm[1]);
		case OpCylinder: return SdCylinder(p, prm[0], prm[1]);
		case OpCone: return SdCone(p, prm[0], prm[1]);
		case OpConinder: return SdConinder(p, prm[0], prm[1], prm[2]);
		case OpPlane: return SdPlane(p, Vec3(prm[0], prm[1], prm[2]));
		default: return 0.0f;
		}
	}

	// The smooth operators are the polynomial blend: h = max(k - |l -+ r|, 0), then
	// min/max(l, r) -+ h*h/4k, evaluated in double as the reference's double literal makes
	// it.  Where the operands are at least k apart (h = 0, nearly everywhere) the double
	// term is +0 and the result is m -+ 0 rounded to float, which one float add or
	// subtract of 0 reproduces exactly (signed zeros included); only k > 0 takes that
	// shortcut, since 0/0 must stay NaN.
	// The double-precision path is kept out of line so the compiler cannot evaluate it
	// speculatively alongside the common shortcut (GB300 issues FP64 at a small fraction
	// of the FP32 rate).
#if defined(__CUDACC__)
	static __host__ __device__ __noinline__
#else
	inline
#endif
	float BlendTermDouble(float m, float h, float k, bool subtract)
	{
		const double q = (double)(h * h) * 0.25 / (double)k;
		return (float)(subtract ? (double)m - q : (double)m + q);
	}

#if defined(__CUDACC__)
	// The blend term's double result rounded to float, computed in float where that is
	// provably the same value (GPU only; the double path stays the reference).
	//
	// With a = hh/4 (exact), q = a/k is taken as qh + ql: qh = RN(a/k), the remainder
	// r = a - qh*k is exact (one fused multiply-add), ql = RN(r/k), so |q - qh - ql| <=
	// 2^-48 |qh|.  TwoSum gives m -+ qh = s + e exactly; t = RN(e -+ ql); TwoSum gives
	// s + t = R + w exactly with R = RN(s + t).  The reference's value d = RN53(m -+ RN53(q))
	// then satisfies |d - (R + w)| <= 2^-46 (|m| + |qh| + |R|) (the two float roundings
	// above at 2^-48 each, the two double roundings at 2^-53), so when |w| plus that bound
	// stays below half the gap around R -- a quarter ulp when |R| is a power of two, where
	// the gap below is half as wide -- RN24(d) = R exactly.  Otherwise, or outside the
	// ranges where the steps above are exact (tiny or huge operands, non-finite values),
	// the caller takes the double path.  Failing the test is rare (about 2^-22 (|m| + |q|)
	// / |R| of the evaluations).
	__device__ __forceinline__ bool BlendTermFloat(float m, float hh, float k, bool subtract, float& out)
	{
		if (!(hh >= 0x1p-100f && hh <= 0x1p100f && k >= 0x1p-100f && k <= 0x1p100f)) return false;
		const float a = hh * 0.25f;
		const float qh = __fdiv_rn(a, k);
		const float aq = fabsf(qh);
		if (!(aq >= 0x1p-100f && aq <= 0x1p100f)) return false;
		const float r = __fmaf_rn(-qh, k, a);
		const float ql = __fdiv_rn(r, k);
		const float b = subtract ? -qh : qh;
		const float bl = subtract ? -ql : ql;
		const float s = __fadd_rn(m, b);
		const float bp = __fsub_rn(s, m);
		const float e = __fadd_rn(__fsub_rn(m, __fsub_rn(s, bp)), __fsub_rn(b, bp));
		const float t = __fadd_rn(e, bl);
		const float R = __fadd_rn(s, t);
		const float tp = __fsub_rn(R, s);
		const float w = __fadd_rn(__fsub_rn(s, __fsub_rn(R, tp)), __fsub_rn(t, tp));
		const uint32_t bits = __float_as_uint(R) & 0x7FFFFFFFu;
		if (bits < (25u << 23) || bits >= (0xFFu << 23)) return false;
		const float ulp = __uint_as_float((bits & 0x7F800000u) - (23u << 23));
		const float half = (bits & 0x007FFFFFu) ? 0.5f * ulp : 0.25f * ulp;
		const float bound = 0x1p-46f * __fadd_rn(__fadd_rn(fabsf(m), aq), fabsf(R));
		if (!(__fadd_rn(fabsf(w), bound) < half)) return false;
		out = R;
		return true;
	}
#endif

	TG_HD float BlendTerm(float m, float h, float k, bool subtract)
	{
		if (h == 0.0f && k > 0.0f) return subtract ? m - 0.0f : m + 0.0f;
#if defined(__CUDA_ARCH__)
		float fast;
		if (BlendTermFloat(m, h * h, k, subtract, fast)) return fast;
#endif
		return BlendTermDouble(m, h, k, subtract);
	}

	TG_HD float SetDistance(uint32_t op, float l, float r, float k)
	{
		switch (op)
		{
		case OpUnion: return fminf(l, r);
		case OpInter: return fmaxf(l, r);
		case OpDiff: return fmaxf(l, -r);
		case OpBlendUnion: return BlendTerm(fminf(l, r), fmaxf(k - fabsf(l - r), 0.0f), k, true);
		case OpBlendInter: return BlendTerm(fmaxf(l, r), fmaxf(k - fabsf(l - r), 0.0f), k, false);
		case OpBlendDiff: return BlendTerm(fmaxf(l, -r), fmaxf(k - fabsf(l + r), 0.0f), k, false);
		default: return 0.0f;
		}
	}
}
