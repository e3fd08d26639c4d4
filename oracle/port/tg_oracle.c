/*
 * Test infrastructure only -- the CPU oracle for the GPU export path (see tg_oracle.h).
 *
 * Each function names the reference file:line it restates.  The float arithmetic keeps
 * the reference's types and operation order, including the places where a double literal
 * promotes a float expression to double (Ellipsoid, the blend operators, Cone).
 */
#define _GNU_SOURCE
#include "tg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

/* ------------------------------------------------------------------------------------ */
/* Tree spec op codes (a postfix construction program; see oracle/ref_harness.cpp).     */
enum
{
	SPEC_SPHERE = 1, SPEC_ELLIPSOID, SPEC_BOX, SPEC_TORUS, SPEC_CYLINDER, SPEC_PLANE, SPEC_CONE, SPEC_CONINDER,
	SPEC_UNION, SPEC_DIFF, SPEC_INTER, SPEC_BUNION, SPEC_BDIFF, SPEC_BINTER, SPEC_FLATE,
	SPEC_MOVE, SPEC_ROTATE, SPEC_SCALE, SPEC_PAINT, SPEC_ALIGN, SPEC_STENCIL, SPEC_TRANSFORM,
};

/* Interpreter op codes: OpcodeT, sdf_evaluator.h:83-107. */
enum
{
	OP_STOP = 0, OP_SPHERE, OP_ELLIPSOID, OP_BOX, OP_TORUS, OP_CYLINDER, OP_CONE, OP_CONINDER, OP_PLANE,
	OP_UNION, OP_INTER, OP_DIFF, OP_BLEND_UNION, OP_BLEND_INTER, OP_BLEND_DIFF, OP_FLATE,
	OP_OFFSET, OP_MATRIX, OP_SCALE_FIELD,
};

/* ------------------------------------------------------------------------------------ */
/* glm-ordered float vector math (glm 0.9.9.8, packed_highp: no SIMD paths).            */
typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;
typedef struct { float w, x, y, z; } qt;

static inline v3 V3(float x, float y, float z) { v3 r = { x, y, z }; return r; }
static inline v2 V2(float x, float y) { v2 r = { x, y }; return r; }
static inline v3 add3(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 muls3(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 divs3(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline v3 abs3(v3 a) { return V3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
/* glm::max/min scalar: (x < y) ? y : x and (y < x) ? y : x (func_common.inl). */
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline v3 gmax3(v3 a, v3 b) { return V3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
static inline v3 gmin3(v3 a, v3 b) { return V3(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
static inline float dot3(v3 a, v3 b) { v3 t = mul3(a, b); return t.x + t.y + t.z; }
static inline float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float len3(v3 a) { return sqrtf(dot3(a, a)); }
static inline float len2(v2 a) { return sqrtf(dot2(a, a)); }
static inline v3 cross3(v3 x, v3 y)
{
	return V3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
/* glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x). */
static inline v3 normalize3(v3 v) { float s = 1.0f / sqrtf(dot3(v, v)); return muls3(v, s); }
/* glm::clamp(x, lo, hi) = min(max(x, lo), hi) with the ternary min/max. */
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
static inline float gsign(float x) { return (float)((0.0f < x) - (x < 0.0f)); }

/* qua * vec3, type_quat.inl:343-350. */
static inline v3 qrot(qt q, v3 v)
{
	v3 qv = V3(q.x, q.y, q.z);
	v3 uv = cross3(qv, v);
	v3 uuv = cross3(qv, uv);
	return add3(v, muls3(add3(muls3(uv, q.w), uuv), 2.0f));
}
/* qua * qua, type_quat.inl:282-292. */
static inline qt qmul(qt p, qt q)
{
	qt r;
	r.w = p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z;
	r.x = p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y;
	r.y = p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z;
	r.z = p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x;
	return r;
}
/* inverse(qua) = conjugate(q) / dot(q, q), quaternion_common.inl:113-122 with the
 * quaternion dot (w*w + x*x) + (y*y + z*z), type_quat.inl:16-23. */
static inline qt qinv(qt q)
{
	float d = (q.w * q.w + q.x * q.x) + (q.y * q.y + q.z * q.z);
	qt r = { q.w / d, -q.x / d, -q.y / d, -q.z / d };
	return r;
}
static inline int qidentity(qt q) { return q.w == 1.0f && q.x == 0.0f && q.y == 0.0f && q.z == 0.0f; }

/* 4x4 column-major matrix, m[c*4 + r]. */
typedef struct { float m[16]; } m4;

static m4 m4_identity(void) { m4 r; memset(&r, 0, sizeof r); r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f; return r; }

/* mat4 * mat4, type_mat4x4.inl:630-648: Result[c] = ((A0*B[c][0] + A1*B[c][1]) + A2*B[c][2]) + A3*B[c][3]. */
static m4 m4_mul(const m4* a, const m4* b)
{
	m4 r;
	for (int c = 0; c < 4; ++c)
	{
		for (int i = 0; i < 4; ++i)
		{
			float t = a->m[0 * 4 + i] * b->m[c * 4 + 0];
			t = t + a->m[1 * 4 + i] * b->m[c * 4 + 1];
			t = t + a->m[2 * 4 + i] * b->m[c * 4 + 2];
			t = t + a->m[3 * 4 + i] * b->m[c * 4 + 3];
			r.m[c * 4 + i] = t;
		}
	}
	return r;
}

/* mat3_cast(quat) widened to mat4, gtc/quaternion.inl:41-72. */
static m4 m4_from_quat(qt q)
{
	m4 r = m4_identity();
	float qxx = q.x * q.x, qyy = q.y * q.y, qzz = q.z * q.z;
	float qxz = q.x * q.z, qxy = q.x * q.y, qyz = q.y * q.z;
	float qwx = q.w * q.x, qwy = q.w * q.y, qwz = q.w * q.z;
	r.m[0] = 1.0f - 2.0f * (qyy + qzz);
	r.m[1] = 2.0f * (qxy + qwz);
	r.m[2] = 2.0f * (qxz - qwy);
	r.m[4] = 2.0f * (qxy - qwz);
	r.m[5] = 1.0f - 2.0f * (qxx + qzz);
	r.m[6] = 2.0f * (qyz + qwx);
	r.m[8] = 2.0f * (qxz + qwy);
	r.m[9] = 2.0f * (qyz - qwx);
	r.m[10] = 1.0f - 2.0f * (qxx + qyy);
	return r;
}

/* The general 4x4 inverse by cofactors, func_matrix.inl compute_inverse<4,4>. */
static m4 m4_inverse(const m4* M)
{
#define E(c, r) (M->m[(c) * 4 + (r)])
	float Coef00 = E(2,2) * E(3,3) - E(3,2) * E(2,3);
	float Coef02 = E(1,2) * E(3,3) - E(3,2) * E(1,3);
	float Coef03 = E(1,2) * E(2,3) - E(2,2) * E(1,3);
	float Coef04 = E(2,1) * E(3,3) - E(3,1) * E(2,3);
	float Coef06 = E(1,1) * E(3,3) - E(3,1) * E(1,3);
	float Coef07 = E(1,1) * E(2,3) - E(2,1) * E(1,3);
	float Coef08 = E(2,1) * E(3,2) - E(3,1) * E(2,2);
	float Coef10 = E(1,1) * E(3,2) - E(3,1) * E(1,2);
	float Coef11 = E(1,1) * E(2,2) - E(2,1) * E(1,2);
	float Coef12 = E(2,0) * E(3,3) - E(3,0) * E(2,3);
	float Coef14 = E(1,0) * E(3,3) - E(3,0) * E(1,3);
	float Coef15 = E(1,0) * E(2,3) - E(2,0) * E(1,3);
	float Coef16 = E(2,0) * E(3,2) - E(3,0) * E(2,2);
	float Coef18 = E(1,0) * E(3,2) - E(3,0) * E(1,2);
	float Coef19 = E(1,0) * E(2,2) - E(2,0) * E(1,2);
	float Coef20 = E(2,0) * E(3,1) - E(3,0) * E(2,1);
	float Coef22 = E(1,0) * E(3,1) - E(3,0) * E(1,1);
	float Coef23 = E(1,0) * E(2,1) - E(2,0) * E(1,1);

	float Fac0[4] = { Coef00, Coef00, Coef02, Coef03 };
	float Fac1[4] = { Coef04, Coef04, Coef06, Coef07 };
	float Fac2[4] = { Coef08, Coef08, Coef10, Coef11 };
	float Fac3[4] = { Coef12, Coef12, Coef14, Coef15 };
	float Fac4[4] = { Coef16, Coef16, Coef18, Coef19 };
	float Fac5[4] = { Coef20, Coef20, Coef22, Coef23 };
	float Vec0[4] = { E(1,0), E(0,0), E(0,0), E(0,0) };
	float Vec1[4] = { E(1,1), E(0,1), E(0,1), E(0,1) };
	float Vec2[4] = { E(1,2), E(0,2), E(0,2), E(0,2) };
	float Vec3[4] = { E(1,3), E(0,3), E(0,3), E(0,3) };
	float Inv0[4], Inv1[4], Inv2[4], Inv3[4];
	for (int i = 0; i < 4; ++i)
	{
		Inv0[i] = Vec1[i] * Fac0[i] - Vec2[i] * Fac1[i] + Vec3[i] * Fac2[i];
		Inv1[i] = Vec0[i] * Fac0[i] - Vec2[i] * Fac3[i] + Vec3[i] * Fac4[i];
		Inv2[i] = Vec0[i] * Fac1[i] - Vec1[i] * Fac3[i] + Vec3[i] * Fac5[i];
		Inv3[i] = Vec0[i] * Fac2[i] - Vec1[i] * Fac4[i] + Vec2[i] * Fac5[i];
	}
	const float SignA[4] = { +1, -1, +1, -1 };
	const float SignB[4] = { -1, +1, -1, +1 };
	m4 Inv;
	for (int i = 0; i < 4; ++i)
	{
		Inv.m[0 * 4 + i] = Inv0[i] * SignA[i];
		Inv.m[1 * 4 + i] = Inv1[i] * SignB[i];
		Inv.m[2 * 4 + i] = Inv2[i] * SignA[i];
		Inv.m[3 * 4 + i] = Inv3[i] * SignB[i];
	}
	float Row0[4] = { Inv.m[0], Inv.m[4], Inv.m[8], Inv.m[12] };
	float Dot0[4];
	for (int i = 0; i < 4; ++i) Dot0[i] = E(0, i) * Row0[i];
	float Dot1 = (Dot0[0] + Dot0[1]) + (Dot0[2] + Dot0[3]);
	float OneOverDeterminant = 1.0f / Dot1;
	for (int i = 0; i < 16; ++i) Inv.m[i] = Inv.m[i] * OneOverDeterminant;
	return Inv;
#undef E
}

/* ------------------------------------------------------------------------------------ */
/* Transform (tangerine/transform.cpp).                                                 */
typedef struct
{
	qt rot;
	v3 trans;
	float scale;
} xform;

static xform xf_identity(void) { xform t = { { 1, 0, 0, 0 }, { 0, 0, 0 }, 1.0f }; return t; }
static void xf_move(xform* t, v3 o) { t->trans = add3(t->trans, o); }                        /* transform.cpp:33 */
static void xf_rotate(xform* t, qt q) { t->trans = qrot(q, t->trans); t->rot = qmul(q, t->rot); } /* :39 */
static void xf_scale(xform* t, float s) { t->trans = muls3(t->trans, s); t->scale = t->scale * s; } /* :46 */
static v3 xf_apply(const xform* t, v3 p) { return add3(qrot(t->rot, muls3(p, t->scale)), t->trans); } /* :62 */
static v3 xf_apply_inv(const xform* t, v3 p) { return divs3(qrot(qinv(t->rot), sub3(p, t->trans)), t->scale); } /* :68 */
static int xf_equal(const xform* a, const xform* b)
{
	return a->rot.w == b->rot.w && a->rot.x == b->rot.x && a->rot.y == b->rot.y && a->rot.z == b->rot.z &&
		a->trans.x == b->trans.x && a->trans.y == b->trans.y && a->trans.z == b->trans.z && a->scale == b->scale;
}
/* ToMatrix = scale_slow(translate(I, T), vec3(S)) * toMat4(R), transform.cpp:52-58. */
static m4 xf_to_matrix(const xform* t)
{
	m4 R = m4_from_quat(t->rot);
	m4 I = m4_identity();
	/* translate: Result[3] = ((m0*v0 + m1*v1) + m2*v2) + m3 */
	m4 T = I;
	for (int i = 0; i < 4; ++i)
	{
		float a = I.m[0 * 4 + i] * t->trans.x;
		a = a + I.m[1 * 4 + i] * t->trans.y;
		a = a + I.m[2 * 4 + i] * t->trans.z;
		a = a + I.m[3 * 4 + i];
		T.m[3 * 4 + i] = a;
	}
	m4 S = m4_identity();
	S.m[0] = t->scale; S.m[5] = t->scale; S.m[10] = t->scale;
	m4 TS = m4_mul(&T, &S);
	return m4_mul(&TS, &R);
}

/* ------------------------------------------------------------------------------------ */
/* AABB (tangerine/aabb.cpp).                                                           */
typedef struct { v3 min, max; } aabb;

static int aabb_degenerate(aabb b)
{
	int anyinf = isinf(b.min.x) || isinf(b.min.y) || isinf(b.min.z) || isinf(b.max.x) || isinf(b.max.y) || isinf(b.max.z);
	int anynan = isnan(b.min.x) || isnan(b.min.y) || isnan(b.min.z) || isnan(b.max.x) || isnan(b.max.y) || isnan(b.max.z);
	int bad = b.max.x <= b.min.x || b.max.y <= b.min.y || b.max.z <= b.min.z;
	return anyinf || anynan || bad;
}
static aabb aabb_bounding_cube(aabb b) /* aabb.cpp:122-139 */
{
	if (aabb_degenerate(b)) { aabb z = { { 0, 0, 0 }, { 0, 0, 0 } }; return z; }
	v3 e = sub3(b.max, b.min);
	float longest = fmaxf(fmaxf(e.x, e.y), e.z);
	v3 pad = mul3(sub3(V3(longest, longest, longest), e), V3(0.5f, 0.5f, 0.5f));
	aabb r = { sub3(b.min, pad), add3(b.max, pad) };
	return r;
}
static float aabb_volume(aabb b)
{
	if (aabb_degenerate(b)) return 0.0f;
	v3 e = sub3(b.max, b.min);
	return e.x * e.y * e.z;
}

/* ------------------------------------------------------------------------------------ */
/* SDFMath (sdf_evaluator.cpp:165-295).                                                  */
static float m_sphere(v3 p, float r) { return len3(p) - r; }
static float m_ellipsoid(v3 p, v3 r)
{
	float k0 = len3(V3(p.x / r.x, p.y / r.y, p.z / r.z));
	v3 rr = mul3(r, r);
	float k1 = len3(V3(p.x / rr.x, p.y / rr.y, p.z / rr.z));
	return (float)((double)k0 * ((double)k0 - 1.0) / (double)k1);
}
static float m_box(v3 p, v3 e)
{
	v3 a = sub3(abs3(p), e);
	return len3(gmax3(a, V3(0, 0, 0))) + fminf(fmaxf(fmaxf(a.x, a.y), a.z), 0.0f);
}
static float m_torus(v3 p, float R, float r)
{
	return len2(V2(len2(V2(p.x, p.y)) - R, p.z)) - r;
}
static float m_cylinder(v3 p, float r, float e)
{
	v2 d = V2(fabsf(len2(V2(p.x, p.y))) - r, fabsf(p.z) - e);
	return fminf(fmaxf(d.x, d.y), 0.0f) + len2(V2(gmax(d.x, 0.0f), gmax(d.y, 0.0f)));
}
static float m_plane(v3 p, v3 n) { return dot3(p, n); }
static float m_cone(v3 p, float tangent, float height)
{
	v2 q = V2(height * tangent, height * -1.0f);
	v2 w = V2(len2(V2(p.x, p.y)), (float)((double)height * -0.5 + (double)p.z));
	float ca = gclamp((float)(dot2(w, q) / dot2(q, q)), 0.0f, 1.0f);
	v2 a = V2(w.x - q.x * ca, w.y - q.y * ca);
	float cb = gclamp((float)(w.x / q.x), 0.0f, 1.0f);
	v2 b = V2(w.x - q.x * cb, w.y - q.y * 1.0f);
	float k = gsign(q.y);
	float d = fminf(dot2(a, a), dot2(b, b));
	float s = fmaxf(k * (w.x * q.y - w.y * q.x), k * (w.y - q.y));
	return sqrtf(d) * gsign(s);
}
static float m_coninder(v3 p, float rl, float rh, float h)
{
	v2 q = V2(len2(V2(p.x, p.y)), p.z);
	v2 k1 = V2(rh, h);
	v2 k2 = V2(rh - rl, (float)(2.0 * (double)h));
	v2 ca = V2(q.x - fminf(q.x, (q.y < 0.0f) ? rl : rh), fabsf(q.y) - h);
	v2 k1q = V2(k1.x - q.x, k1.y - q.y);
	float c = gclamp(dot2(k1q, k2) / dot2(k2, k2), 0.0f, 1.0f);
	v2 qk = V2(q.x - k1.x, q.y - k1.y);
	v2 cb = V2(qk.x + k2.x * c, qk.y + k2.y * c);
	float s = (cb.x < 0.0f && ca.y < 0.0f) ? -1.0f : 1.0f;
	return s * sqrtf(fminf(dot2(ca, ca), dot2(cb, cb)));
}
static float m_union(float l, float r) { return fminf(l, r); }
static float m_inter(float l, float r) { return fmaxf(l, r); }
static float m_diff(float l, float r) { return fmaxf(l, -r); }
static float m_blend_union(float l, float r, float k)
{
	float h = fmaxf(k - fabsf(l - r), 0.0f);
	return (float)((double)fminf(l, r) - (double)(h * h) * 0.25 / (double)k);
}
static float m_blend_inter(float l, float r, float k)
{
	float h = fmaxf(k - fabsf(l - r), 0.0f);
	return (float)((double)fmaxf(l, r) + (double)(h * h) * 0.25 / (double)k);
}
static float m_blend_diff(float l, float r, float k)
{
	float h = fmaxf(k - fabsf(l + r), 0.0f);
	return (float)((double)fmaxf(l, -r) + (double)(h * h) * 0.25 / (double)k);
}

static float brush_math(int op, const float* prm, v3 p)
{
	switch (op)
	{
	case OP_SPHERE: return m_sphere(p, prm[0]);
	case OP_ELLIPSOID: return m_ellipsoid(p, V3(prm[0], prm[1], prm[2]));
	case OP_BOX: return m_box(p, V3(prm[0], prm[1], prm[2]));
	case OP_TORUS: return m_torus(p, prm[0], prm[1]);
	case OP_CYLINDER: return m_cylinder(p, prm[0], prm[1]);
	case OP_CONE: return m_cone(p, prm[0], prm[1]);
	case OP_CONINDER: return m_coninder(p, prm[0], prm[1], prm[2]);
	case OP_PLANE: return m_plane(p, V3(prm[0], prm[1], prm[2]));
	default: return 0.0f;
	}
}
static float set_math(int op, float l, float r, float k)
{
	switch (op)
	{
	case OP_UNION: return m_union(l, r);
	case OP_INTER: return m_inter(l, r);
	case OP_DIFF: return m_diff(l, r);
	case OP_BLEND_UNION: return m_blend_union(l, r, k);
	case OP_BLEND_INTER: return m_blend_inter(l, r, k);
	case OP_BLEND_DIFF: return m_blend_diff(l, r, k);
	default: return 0.0f;
	}
}
static int brush_param_count(int op)
{
	switch (op)
	{
	case OP_SPHERE: return 1;
	case OP_TORUS: case OP_CYLINDER: case OP_CONE: return 2;
	default: return 3;
	}
}

/* ------------------------------------------------------------------------------------ */
/* CSG nodes (sdf_evaluator.cpp:432-1160).  Nodes are immutable once built, except for   */
/* the mutators applied while a spec is being executed; clipped trees share subtrees.   */
enum { K_BRUSH, K_SET, K_FLATE, K_STENCIL };

typedef struct node node;
struct node
{
	int kind;
	int op;               /* interpreter opcode of the brush or set operator */
	int stack_size;
	/* brush */
	float prm[3];
	aabb brush_aabb;
	xform xf;
	int material;         /* -1: none (default white) */
	/* set / flate / stencil */
	node* lhs;
	node* rhs;
	float threshold;      /* set: blend threshold; flate: radius */
	node* mask;
	int negative;
};

typedef struct arena_block { struct arena_block* next; size_t used; char data[1 << 16]; } arena_block;
typedef struct { arena_block* head; } arena;

static void* arena_alloc(arena* a, size_t n)
{
	n = (n + 15) & ~(size_t)15;
	if (!a->head || a->head->used + n > sizeof a->head->data)
	{
		arena_block* b = (arena_block*)malloc(sizeof(arena_block));
		b->next = a->head;
		b->used = 0;
		a->head = b;
	}
	void* p = a->head->data + a->head->used;
	a->head->used += n;
	return p;
}
static void arena_free(arena* a)
{
	arena_block* b = a->head;
	while (b) { arena_block* n = b->next; free(b); b = n; }
	a->head = NULL;
}

typedef struct { float rgb[3]; } material;

struct tgo_tree
{
	arena mem;
	node* root;
	material* materials;
	int material_count;
	int material_capacity;
	int owns_materials;
};

static node* new_node(arena* a) { node* n = (node*)arena_alloc(a, sizeof(node)); memset(n, 0, sizeof *n); n->material = -1; return n; }

static node* make_brush(arena* a, int op, const float* prm, aabb box)
{
	node* n = new_node(a);
	n->kind = K_BRUSH;
	n->op = op;
	for (int i = 0; i < brush_param_count(op); ++i) n->prm[i] = prm[i];
	n->brush_aabb = box;
	n->xf = xf_identity();
	n->stack_size = 1;
	return n;
}

/* SetNode ctor, sdf_evaluator.cpp:737-772: non-Diff operators swap so the tree leans left. */
static node* make_set(arena* a, int op, node* l, node* r, float k)
{
	node* n = new_node(a);
	n->kind = K_SET;
	n->op = op;
	int is_diff = (op == OP_DIFF || op == OP_BLEND_DIFF);
	if (!is_diff && r->stack_size > l->stack_size) { node* t = l; l = r; r = t; }
	n->lhs = l;
	n->rhs = r;
	n->threshold = k;
	int s = r->stack_size + 1;
	n->stack_size = l->stack_size > s ? l->stack_size : s;
	return n;
}
static node* make_flate(arena* a, node* child, float radius)
{
	node* n = new_node(a);
	n->kind = K_FLATE;
	n->lhs = child;
	n->threshold = radius;
	n->stack_size = child->stack_size;
	return n;
}
static node* make_stencil(arena* a, node* child, node* mask, int mat, int negative)
{
	node* n = new_node(a);
	n->kind = K_STENCIL;
	n->lhs = child;
	n->mask = mask;
	n->material = mat;
	n->negative = negative;
	n->stack_size = child->stack_size;
	return n;
}

static aabb sym_bounds(v3 h) { aabb b = { V3(h.x * -1.0f, h.y * -1.0f, h.z * -1.0f), h }; return b; }

/* SDF:: constructors, sdf_evaluator.cpp:1206-1317. */
static node* make_primitive(arena* a, int spec_op, const float* P)
{
	float prm[3];
	switch (spec_op)
	{
	case SPEC_SPHERE: prm[0] = P[0]; return make_brush(a, OP_SPHERE, prm, sym_bounds(V3(P[0], P[0], P[0])));
	case SPEC_ELLIPSOID: memcpy(prm, P, 12); return make_brush(a, OP_ELLIPSOID, prm, sym_bounds(V3(P[0], P[1], P[2])));
	case SPEC_BOX: memcpy(prm, P, 12); return make_brush(a, OP_BOX, prm, sym_bounds(V3(P[0], P[1], P[2])));
	case SPEC_TORUS:
	{
		prm[0] = P[0]; prm[1] = P[1];
		float r = P[0] + P[1];
		return make_brush(a, OP_TORUS, prm, sym_bounds(V3(r, r, P[1])));
	}
	case SPEC_CYLINDER: prm[0] = P[0]; prm[1] = P[1]; return make_brush(a, OP_CYLINDER, prm, sym_bounds(V3(P[0], P[0], P[1])));
	case SPEC_PLANE:
	{
		v3 n = normalize3(V3(P[0], P[1], P[2]));
		prm[0] = n.x; prm[1] = n.y; prm[2] = n.z;
		aabb b = sym_bounds(V3(INFINITY, INFINITY, INFINITY));
		if (n.x == -1.0f) b.min.x = 0.0f;
		else if (n.x == 1.0f) b.max.x = 0.0f;
		else if (n.y == -1.0f) b.min.y = 0.0f;
		else if (n.y == 1.0f) b.max.y = 0.0f;
		else if (n.z == -1.0f) b.min.z = 0.0f;
		else if (n.z == 1.0f) b.max.z = 0.0f;
		return make_brush(a, OP_PLANE, prm, b);
	}
	case SPEC_CONE:
	{
		float tangent = P[0] / P[1];
		prm[0] = tangent; prm[1] = P[1];
		return make_brush(a, OP_CONE, prm, sym_bounds(V3(P[0], P[0], (float)((double)P[1] * 0.5))));
	}
	case SPEC_CONINDER:
	{
		float half = (float)((double)P[2] * 0.5);
		prm[0] = P[0]; prm[1] = P[1]; prm[2] = half;
		float mr = fmaxf(P[0], P[1]);
		return make_brush(a, OP_CONINDER, prm, sym_bounds(V3(mr, mr, half)));
	}
	}
	return NULL;
}

static float node_eval(const node* n, v3 p);

/* Mutators (sdf_evaluator.cpp:509-530, 637-658, 926-949, 1105-1123).  Applied in place
 * while a spec runs, before any subtree is shared. */
static void node_move(node* n, v3 o)
{
	switch (n->kind)
	{
	case K_BRUSH: xf_move(&n->xf, o); break;
	case K_SET: node_move(n->lhs, o); node_move(n->rhs, o); break;
	case K_FLATE: node_move(n->lhs, o); break;
	case K_STENCIL: node_move(n->lhs, o); node_move(n->mask, o); break;
	}
}
static void node_rotate(node* n, qt q)
{
	switch (n->kind)
	{
	case K_BRUSH: xf_rotate(&n->xf, q); break;
	case K_SET: node_rotate(n->lhs, q); node_rotate(n->rhs, q); break;
	case K_FLATE: node_rotate(n->lhs, q); break;
	case K_STENCIL: node_rotate(n->lhs, q); node_rotate(n->mask, q); break;
	}
}
static void node_scale(node* n, float s)
{
	switch (n->kind)
	{
	case K_BRUSH: xf_scale(&n->xf, s); break;
	case K_SET: n->threshold = n->threshold * s; node_scale(n->lhs, s); node_scale(n->rhs, s); break;
	case K_FLATE: node_scale(n->lhs, s); break;
	case K_STENCIL: node_scale(n->lhs, s); node_scale(n->mask, s); break;
	}
}
static int node_has_paint(const node* n)
{
	switch (n->kind)
	{
	case K_BRUSH: return n->material >= 0;
	case K_SET: return node_has_paint(n->lhs) || node_has_paint(n->rhs);
	case K_FLATE: return node_has_paint(n->lhs);
	default: return 1;
	}
}
static void node_apply_material(node* n, int mat, int force)
{
	switch (n->kind)
	{
	case K_BRUSH: if (n->material < 0 || force) n->material = mat; break;
	case K_SET: node_apply_material(n->lhs, mat, force); node_apply_material(n->rhs, mat, force); break;
	case K_FLATE: node_apply_material(n->lhs, mat, force); break;
	default: break; /* StencilMaskNode::ApplyMaterial is a no-op */
	}
}
static int node_finite(const node* n)
{
	switch (n->kind)
	{
	case K_BRUSH:
		return !(isinf(n->brush_aabb.min.x) || isinf(n->brush_aabb.min.y) || isinf(n->brush_aabb.min.z) ||
			isinf(n->brush_aabb.max.x) || isinf(n->brush_aabb.max.y) || isinf(n->brush_aabb.max.z));
	case K_SET: return node_finite(n->lhs) || node_finite(n->rhs);
	default: return node_finite(n->lhs);
	}
}
static int node_leaf_count(const node* n)
{
	switch (n->kind)
	{
	case K_BRUSH: return 1;
	case K_SET: return node_leaf_count(n->lhs) + node_leaf_count(n->rhs);
	default: return node_leaf_count(n->lhs);
	}
}

/* EvaluatorTransform::Apply, sdf_evaluator.cpp:367-406. */
static aabb xf_apply_bounds(const xform* t, aabb in)
{
	if (qidentity(t->rot))
	{
		aabb r = { add3(muls3(in.min, t->scale), t->trans), add3(muls3(in.max, t->scale), t->trans) };
		return r;
	}
	v3 A = in.min, B = in.max;
	v3 pts[7] = { B, V3(B.x, A.y, A.z), V3(A.x, B.y, A.z), V3(A.x, A.y, B.z), V3(A.x, B.y, B.z), V3(B.x, A.y, B.z), V3(B.x, B.y, A.z) };
	aabb r;
	r.min = xf_apply(t, A);
	r.max = r.min;
	for (int i = 0; i < 7; ++i)
	{
		v3 q = xf_apply(t, pts[i]);
		r.min = gmin3(r.min, q);
		r.max = gmax3(r.max, q);
	}
	return r;
}

static aabb node_bounds(const node* n, int inner)
{
	switch (n->kind)
	{
	case K_BRUSH: return xf_apply_bounds(&n->xf, n->brush_aabb);
	case K_STENCIL: return node_bounds(n->lhs, inner);
	case K_FLATE:
	{
		/* FlateNode::Bounds, sdf_evaluator.cpp:1082-1096: Max += vec3(R*2), Min -= vec3(R*2) */
		aabb b = node_bounds(n->lhs, inner);
		float r2 = n->threshold * 2.0f;
		b.max = add3(b.max, V3(r2, r2, r2));
		b.min = sub3(b.min, V3(r2, r2, r2));
		return b;
	}
	case K_SET:
	{
		/* SetNode::Bounds / InnerBounds, sdf_evaluator.cpp:857-913 */
		aabb L = node_bounds(n->lhs, inner), R = node_bounds(n->rhs, inner), c;
		if (n->op == OP_UNION || n->op == OP_BLEND_UNION) { c.min = gmin3(L.min, R.min); c.max = gmax3(L.max, R.max); }
		else if (n->op == OP_DIFF || n->op == OP_BLEND_DIFF) { c = L; }
		else { c.min = gmax3(L.min, R.min); c.max = gmin3(L.max, R.max); }
		int blend = (n->op == OP_BLEND_UNION || n->op == OP_BLEND_INTER || n->op == OP_BLEND_DIFF);
		if (blend && !inner)
		{
			float k = n->threshold;
			aabb lim;
			lim.min = sub3(gmax3(L.min, R.min), V3(k, k, k));
			lim.max = add3(gmin3(L.max, R.max), V3(k, k, k));
			c.min = gmin3(c.min, lim.min);
			c.max = gmax3(c.max, lim.max);
		}
		return c;
	}
	}
	aabb z = { { 0, 0, 0 }, { 0, 0, 0 } };
	return z;
}

/* Virtual SDFNode::Eval (sdf_evaluator.cpp:463-466, 598-601, 774-780, 1059-1062). */
static float node_eval(const node* n, v3 p)
{
	switch (n->kind)
	{
	case K_BRUSH: return brush_math(n->op, n->prm, xf_apply_inv(&n->xf, p)) * n->xf.scale;
	case K_SET: return set_math(n->op, node_eval(n->lhs, p), node_eval(n->rhs, p), n->threshold);
	case K_FLATE: return node_eval(n->lhs, p) - n->threshold;
	case K_STENCIL: return node_eval(n->lhs, p);
	}
	return 0.0f;
}

/* Clip (sdf_evaluator.cpp:468-478, 603-615, 782-850, 1064-1075). */
static node* node_clip(arena* a, node* n, v3 p, float radius)
{
	switch (n->kind)
	{
	case K_BRUSH:
		return node_eval(n, p) <= radius ? n : NULL;
	case K_STENCIL:
	{
		node* c = node_clip(a, n->lhs, p, radius);
		return c ? make_stencil(a, c, n->mask, n->material, n->negative) : NULL;
	}
	case K_FLATE:
		if (node_eval(n, p) <= radius)
		{
			node* c = node_clip(a, n->lhs, p, radius + n->threshold);
			return c ? make_flate(a, c, n->threshold) : NULL;
		}
		return NULL;
	case K_SET:
	{
		if (!(node_eval(n, p) <= radius)) return NULL;
		int blend = (n->op == OP_BLEND_UNION || n->op == OP_BLEND_INTER || n->op == OP_BLEND_DIFF);
		int family_union = (n->op == OP_UNION || n->op == OP_BLEND_UNION);
		int family_diff = (n->op == OP_DIFF || n->op == OP_BLEND_DIFF);
		if (blend)
		{
			float wide = radius + n->threshold;
			node* l = node_clip(a, n->lhs, p, wide);
			node* r = node_clip(a, n->rhs, p, wide);
			if (l && r) return make_set(a, n->op, l, r, n->threshold);
			if (!family_union && !family_diff) return NULL;
		}
		node* l = node_clip(a, n->lhs, p, radius);
		node* r = node_clip(a, n->rhs, p, radius);
		if (l && r) return make_set(a, n->op, l, r, n->threshold);
		if (family_union) return l ? l : r;
		if (family_diff) return l;
		return NULL;
	}
	}
	return NULL;
}

/* operator== (sdf_evaluator.cpp:564-579, 696-709, 1029-1037, 1150-1154). */
static int node_equal(const node* a, const node* b)
{
	if (a == b) return 1;
	if (a->kind != b->kind) return 0;
	switch (a->kind)
	{
	case K_BRUSH:
		if (a->op != b->op || a->material != b->material || !xf_equal(&a->xf, &b->xf)) return 0;
		for (int i = 0; i < brush_param_count(a->op); ++i) if (a->prm[i] != b->prm[i]) return 0;
		return 1;
	case K_SET:
		return a->op == b->op && a->threshold == b->threshold && node_equal(a->lhs, b->lhs) && node_equal(a->rhs, b->rhs);
	case K_FLATE:
		return a->threshold == b->threshold && node_equal(a->lhs, b->lhs);
	case K_STENCIL:
		return a->negative == b->negative && a->material == b->material && node_equal(a->lhs, b->lhs) && node_equal(a->mask, b->mask);
	}
	return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Program compilation (sdf_evaluator.cpp:409-429, 495-507, 632-635, 915-924, 1098-1103). */
typedef struct { uint32_t* w; int n, cap; } words;

static void push_word(words* b, uint32_t v)
{
	if (b->n == b->cap) { b->cap = b->cap ? b->cap * 2 : 256; b->w = (uint32_t*)realloc(b->w, (size_t)b->cap * 4); }
	b->w[b->n++] = v;
}
static void push_float(words* b, float f) { uint32_t u; memcpy(&u, &f, 4); push_word(b, u); }

static void node_compile(const node* n, words* b)
{
	switch (n->kind)
	{
	case K_BRUSH:
	{
		const xform* t = &n->xf;
		int has_rot = !qidentity(t->rot);
		int has_scale = t->scale != 1.0f;
		int has_trans = !(t->trans.x == 0.0f && t->trans.y == 0.0f && t->trans.z == 0.0f);
		if (has_rot || has_scale)
		{
			m4 m = xf_to_matrix(t);
			m4 inv = m4_inverse(&m);
			push_word(b, OP_MATRIX);
			for (int i = 0; i < 16; ++i) push_float(b, inv.m[i]);
		}
		else if (has_trans)
		{
			push_word(b, OP_OFFSET);
			push_float(b, -t->trans.x); push_float(b, -t->trans.y); push_float(b, -t->trans.z);
		}
		push_word(b, (uint32_t)n->op);
		for (int i = 0; i < brush_param_count(n->op); ++i) push_float(b, n->prm[i]);
		if (t->scale != 1.0f)
		{
			push_word(b, OP_SCALE_FIELD);
			push_float(b, t->scale);
		}
		break;
	}
	case K_SET:
		node_compile(n->lhs, b);
		node_compile(n->rhs, b);
		push_word(b, (uint32_t)n->op);
		if (n->op == OP_BLEND_UNION || n->op == OP_BLEND_INTER || n->op == OP_BLEND_DIFF) push_float(b, n->threshold);
		break;
	case K_FLATE:
		node_compile(n->lhs, b);
		push_word(b, OP_FLATE);
		push_float(b, n->threshold);
		break;
	case K_STENCIL:
		node_compile(n->lhs, b);
		break;
	}
}

static inline float wf(const uint32_t* w, int i) { float f; memcpy(&f, &w[i], 4); return f; }

/* SDFInterpreter::Eval, sdf_evaluator.cpp:1386-1605. */
static float interp_eval(const uint32_t* w, int n, int stack_size, v3 ep)
{
	float stack_local[64];
	float* stack = stack_size <= 64 ? stack_local : (float*)malloc(sizeof(float) * (size_t)stack_size);
	int sp = 0;
	int pc = 0;
	v3 p = ep;
	float result = 0.0f;
	while (pc < n)
	{
		uint32_t op = w[pc++];
		switch (op)
		{
		case OP_STOP: result = stack[sp - 1]; goto done;
		case OP_SPHERE: case OP_ELLIPSOID: case OP_BOX: case OP_TORUS: case OP_CYLINDER: case OP_CONE: case OP_CONINDER: case OP_PLANE:
		{
			float prm[3];
			int c = brush_param_count((int)op);
			for (int i = 0; i < c; ++i) prm[i] = wf(w, pc + i);
			pc += c;
			stack[sp++] = brush_math((int)op, prm, p);
			p = ep;
			break;
		}
		case OP_UNION: case OP_INTER: case OP_DIFF:
		{
			float r = stack[--sp];
			float l = stack[--sp];
			stack[sp++] = set_math((int)op, l, r, 0.0f);
			break;
		}
		case OP_BLEND_UNION: case OP_BLEND_INTER: case OP_BLEND_DIFF:
		{
			float r = stack[--sp];
			float l = stack[--sp];
			float k = wf(w, pc++);
			stack[sp++] = set_math((int)op, l, r, k);
			break;
		}
		case OP_FLATE: stack[sp - 1] = stack[sp - 1] - wf(w, pc++); break;
		case OP_OFFSET: p = add3(ep, V3(wf(w, pc), wf(w, pc + 1), wf(w, pc + 2))); pc += 3; break;
		case OP_MATRIX:
		{
			/* (M * vec4(p, 1)).xyz = (m0*x + m1*y) + (m2*z + m3*1), type_mat4x4.inl */
			float r3[3];
			for (int i = 0; i < 3; ++i)
			{
				float a0 = wf(w, pc + 0 + i) * ep.x;
				float a1 = wf(w, pc + 4 + i) * ep.y;
				float a2 = wf(w, pc + 8 + i) * ep.z;
				float a3 = wf(w, pc + 12 + i) * 1.0f;
				r3[i] = (a0 + a1) + (a2 + a3);
			}
			p = V3(r3[0], r3[1], r3[2]);
			pc += 16;
			break;
		}
		case OP_SCALE_FIELD: stack[sp - 1] = stack[sp - 1] * wf(w, pc++); break;
		default: goto done;
		}
	}
done:
	if (stack != stack_local) free(stack);
	return result;
}

/* ------------------------------------------------------------------------------------ */
/* Materials: GetMaterial (sdf_evaluator.cpp:537-547, 666-679, 957-1012, 1130-1133).     */
static int node_material(const node* n, v3 p)
{
	switch (n->kind)
	{
	case K_BRUSH: return n->material;
	case K_FLATE: return node_material(n->lhs, p);
	case K_STENCIL:
	{
		int interior = node_eval(n->mask, p) < 0.0f;
		return (interior == n->negative) ? n->material : node_material(n->lhs, p);
	}
	case K_SET:
	{
		if (n->op == OP_DIFF || n->op == OP_BLEND_DIFF) return node_material(n->lhs, p);
		float el = node_eval(n->lhs, p);
		float er = node_eval(n->rhs, p);
		float d = set_math(n->op, el, er, n->threshold);
		int blend = (n->op == OP_BLEND_UNION || n->op == OP_BLEND_INTER);
		int take_left = blend ? (fabsf(el - d) <= fabsf(er - d)) : (d == el);
		if (n->op == OP_UNION || n->op == OP_BLEND_UNION)
		{
			return take_left ? node_material(n->lhs, p) : node_material(n->rhs, p);
		}
		int ml = node_material(n->lhs, p);
		int mr = node_material(n->rhs, p);
		int lv = node_has_paint(n->lhs), rv = node_has_paint(n->rhs);
		if (lv && rv) return take_left ? ml : mr;
		if (lv) return ml;
		return mr;
	}
	}
	return -1;
}

static void color_bytes(const tgo_tree* t, int mat, uint8_t* out)
{
	/* Default material is white (sdf_evaluator.cpp:34-38); 0xFF * c truncates (export.cpp:303-311). */
	float c[3] = { 1.0f, 1.0f, 1.0f };
	if (mat >= 0) { c[0] = t->materials[mat].rgb[0]; c[1] = t->materials[mat].rgb[1]; c[2] = t->materials[mat].rgb[2]; }
	for (int i = 0; i < 3; ++i) out[i] = (uint8_t)(255.0f * c[i]);
}

/* SDFNode::Gradient, sdf_evaluator.cpp:298-333 (tetrahedral, h = 1e-4). */
static v3 node_gradient(const node* n, v3 p)
{
	const float h = 0.0001f;
	v3 xyy = V3(h, -h, -h), yyx = V3(-h, -h, h), yxy = V3(-h, h, -h), xxx = V3(h, h, h);
	v3 g = muls3(xyy, node_eval(n, add3(p, xyy)));
	g = add3(g, muls3(yyx, node_eval(n, add3(p, yyx))));
	g = add3(g, muls3(yxy, node_eval(n, add3(p, yxy))));
	g = add3(g, muls3(xxx, node_eval(n, add3(p, xxx))));
	float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
	if (ls == 0.0f)
	{
		float d = node_eval(n, p);
		return normalize3(V3(node_eval(n, add3(p, xyy)) - d, node_eval(n, add3(p, yxy)) - d, node_eval(n, add3(p, yyx)) - d));
	}
	return divs3(g, sqrtf(ls));
}

/* ------------------------------------------------------------------------------------ */
/* Spec execution.                                                                       */
static int spec_arity(int op)
{
	switch (op)
	{
	case SPEC_SPHERE: return 1;
	case SPEC_ELLIPSOID: case SPEC_BOX: case SPEC_PLANE: case SPEC_CONINDER: return 3;
	case SPEC_TORUS: case SPEC_CYLINDER: case SPEC_CONE: return 2;
	case SPEC_UNION: case SPEC_DIFF: case SPEC_INTER: return 0;
	case SPEC_BUNION: case SPEC_BDIFF: case SPEC_BINTER: case SPEC_FLATE: return 1;
	case SPEC_MOVE: case SPEC_PAINT: case SPEC_ALIGN: return 3;
	case SPEC_ROTATE: case SPEC_STENCIL: return 4;
	case SPEC_SCALE: return 1;
	case SPEC_TRANSFORM: return 8;
	default: return -1;
	}
}

static int add_material(tgo_tree* t, const float* rgb)
{
	if (t->material_count == t->material_capacity)
	{
		t->material_capacity = t->material_capacity ? t->material_capacity * 2 : 64;
		t->materials = (material*)realloc(t->materials, sizeof(material) * (size_t)t->material_capacity);
	}
	memcpy(t->materials[t->material_count].rgb, rgb, 12);
	return t->material_count++;
}

tgo_tree* tgo_build(const float* spec, int count)
{
	tgo_tree* t = (tgo_tree*)calloc(1, sizeof(tgo_tree));
	t->owns_materials = 1;
	node** stack = (node**)malloc(sizeof(node*) * (size_t)(count + 1));
	int sp = 0, i = 0, ok = 1;
	while (i < count && ok)
	{
		int op = (int)spec[i++];
		int ar = spec_arity(op);
		if (ar < 0 || i + ar > count) { ok = 0; break; }
		const float* P = spec + i;
		i += ar;
		switch (op)
		{
		case SPEC_SPHERE: case SPEC_ELLIPSOID: case SPEC_BOX: case SPEC_TORUS: case SPEC_CYLINDER:
		case SPEC_PLANE: case SPEC_CONE: case SPEC_CONINDER:
			stack[sp++] = make_primitive(&t->mem, op, P);
			break;
		case SPEC_UNION: case SPEC_DIFF: case SPEC_INTER: case SPEC_BUNION: case SPEC_BDIFF: case SPEC_BINTER:
		{
			if (sp < 2) { ok = 0; break; }
			node* r = stack[--sp];
			node* l = stack[--sp];
			static const int map[] = { OP_UNION, OP_DIFF, OP_INTER, OP_BLEND_UNION, OP_BLEND_DIFF, OP_BLEND_INTER };
			float k = (op >= SPEC_BUNION) ? P[0] : 0.0f;
			stack[sp++] = make_set(&t->mem, map[op - SPEC_UNION], l, r, k);
			break;
		}
		case SPEC_FLATE:
			if (sp < 1) { ok = 0; break; }
			stack[sp - 1] = make_flate(&t->mem, stack[sp - 1], P[0]);
			break;
		case SPEC_MOVE: if (sp < 1) { ok = 0; break; } node_move(stack[sp - 1], V3(P[0], P[1], P[2])); break;
		case SPEC_ROTATE:
		{
			if (sp < 1) { ok = 0; break; }
			qt q = { P[3], P[0], P[1], P[2] };
			node_rotate(stack[sp - 1], q);
			break;
		}
		case SPEC_SCALE: if (sp < 1) { ok = 0; break; } node_scale(stack[sp - 1], P[0]); break;
		case SPEC_PAINT:
			if (sp < 1) { ok = 0; break; }
			node_apply_material(stack[sp - 1], add_material(t, P), 0);
			break;
		case SPEC_ALIGN:
		{
			/* SDF::Align, sdf_evaluator.cpp:1171-1177: mix(min, max, a) = min*(1-a) + max*a */
			if (sp < 1) { ok = 0; break; }
			v3 al = add3(mul3(V3(P[0], P[1], P[2]), V3(0.5f, 0.5f, 0.5f)), V3(0.5f, 0.5f, 0.5f));
			aabb b = node_bounds(stack[sp - 1], 1);
			v3 one_minus = sub3(V3(1, 1, 1), al);
			v3 mixed = add3(mul3(b.min, one_minus), mul3(b.max, al));
			node_move(stack[sp - 1], mul3(mixed, V3(-1.0f, -1.0f, -1.0f)));
			break;
		}
		case SPEC_TRANSFORM:
			/* a brush's whole transform as it is: rotation (w x y z), translation, scale */
			if (sp < 1 || stack[sp - 1]->kind != K_BRUSH) { ok = 0; break; }
			stack[sp - 1]->xf.rot.w = P[0]; stack[sp - 1]->xf.rot.x = P[1];
			stack[sp - 1]->xf.rot.y = P[2]; stack[sp - 1]->xf.rot.z = P[3];
			stack[sp - 1]->xf.trans = V3(P[4], P[5], P[6]);
			stack[sp - 1]->xf.scale = P[7];
			break;
		case SPEC_STENCIL:
		{
			if (sp < 2) { ok = 0; break; }
			node* mask = stack[--sp];
			node* child = stack[--sp];
			stack[sp++] = make_stencil(&t->mem, child, mask, add_material(t, P + 1), P[0] != 0.0f);
			break;
		}
		default: ok = 0; break;
		}
	}
	if (!ok || sp != 1) { free(stack); arena_free(&t->mem); free(t->materials); free(t); return NULL; }
	t->root = stack[0];
	free(stack);
	return t;
}

void tgo_free(tgo_tree* t)
{
	if (!t) return;
	arena_free(&t->mem);
	if (t->owns_materials) free(t->materials);
	free(t);
}
void tgo_free_buffer(void* b) { free(b); }

int tgo_stack_size(tgo_tree* t) { return t->root->stack_size; }
int tgo_has_paint(tgo_tree* t) { return node_has_paint(t->root); }
int tgo_has_finite_bounds(tgo_tree* t) { return node_finite(t->root); }
int tgo_leaf_count(tgo_tree* t) { return node_leaf_count(t->root); }
void tgo_bounds(tgo_tree* t, float* o, int inner)
{
	aabb b = node_bounds(t->root, inner);
	o[0] = b.min.x; o[1] = b.min.y; o[2] = b.min.z; o[3] = b.max.x; o[4] = b.max.y; o[5] = b.max.z;
}
void tgo_eval(tgo_tree* t, int64_t n, const float* p, float* o)
{
	for (int64_t i = 0; i < n; ++i) o[i] = node_eval(t->root, V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]));
}
void tgo_gradient(tgo_tree* t, int64_t n, const float* p, float* o)
{
	for (int64_t i = 0; i < n; ++i)
	{
		v3 g = node_gradient(t->root, V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]));
		o[i * 3] = g.x; o[i * 3 + 1] = g.y; o[i * 3 + 2] = g.z;
	}
}
void tgo_color(tgo_tree* t, int64_t n, const float* p, uint8_t* o)
{
	for (int64_t i = 0; i < n; ++i) color_bytes(t, node_material(t->root, V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2])), o + i * 3);
}
int tgo_compile(tgo_tree* t, uint32_t* out, int cap)
{
	words b = { 0, 0, 0 };
	node_compile(t->root, &b);
	push_word(&b, OP_STOP);
	for (int i = 0; i < b.n && i < cap; ++i) out[i] = b.w[i];
	int n = b.n;
	free(b.w);
	return n;
}
void tgo_interp_eval(tgo_tree* t, int64_t n, const float* p, float* o)
{
	words b = { 0, 0, 0 };
	node_compile(t->root, &b);
	push_word(&b, OP_STOP);
	for (int64_t i = 0; i < n; ++i) o[i] = interp_eval(b.w, b.n, t->root->stack_size, V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]));
	free(b.w);
}
tgo_tree* tgo_clip(tgo_tree* t, float x, float y, float z, float r)
{
	tgo_tree* c = (tgo_tree*)calloc(1, sizeof(tgo_tree));
	c->root = node_clip(&c->mem, t->root, V3(x, y, z), r);
	c->materials = t->materials;
	c->material_count = t->material_count;
	c->owns_materials = 0;
	if (!c->root) { arena_free(&c->mem); free(c); return NULL; }
	return c;
}
int tgo_equal(tgo_tree* a, tgo_tree* b) { return node_equal(a->root, b->root); }

/* ------------------------------------------------------------------------------------ */
/* SDFOctree (sdf_evaluator.cpp:1609-2005).                                               */
typedef struct onode onode;
struct onode
{
	aabb bounds;
	v3 pivot;
	int terminus;
	int incomplete;
	int evaluator_leaves;
	node* evaluator;
	onode* children[8];
	words program;
	int stack_size;
};

struct tgo_octree
{
	arena mem;
	tgo_tree* tree;
	onode* root;
	float target;
};

static void onode_destroy(onode* o)
{
	if (!o) return;
	for (int i = 0; i < 8; ++i) onode_destroy(o->children[i]);
	free(o->program.w);
	free(o);
}

static void octree_populate(tgo_octree* T, onode* o, int coalesce, int depth, int max_depth);

static onode* octree_node(tgo_octree* T, node* in_eval, aabb bounds, int coalesce, int depth, int max_depth)
{
	onode* o = (onode*)calloc(1, sizeof(onode));
	o->bounds = bounds;
	v3 e = sub3(bounds.max, bounds.min);
	float span = fmaxf(fmaxf(e.x, e.y), e.z);
	float half = (float)((double)span * 0.5);
	o->pivot = add3(V3(half, half, half), bounds.min);
	float radius = (float)((double)len3(V3(span, span, span)) * 0.5);
	o->evaluator = node_clip(&T->mem, in_eval, o->pivot, radius);
	o->evaluator_leaves = o->evaluator ? node_leaf_count(o->evaluator) : 0;
	o->terminus = span <= T->target || o->evaluator == NULL;
	if (!o->terminus)
	{
		o->incomplete = 1;
		if (coalesce || max_depth == -1 || depth < max_depth) octree_populate(T, o, coalesce, depth, max_depth);
	}
	if (o->evaluator)
	{
		node_compile(o->evaluator, &o->program);
		push_word(&o->program, OP_STOP);
		o->stack_size = o->evaluator->stack_size;
	}
	return o;
}

static void octree_populate(tgo_octree* T, onode* o, int coalesce, int depth, int max_depth)
{
	if (!o->incomplete) return;
	o->incomplete = 0;
	int uniform = 1, penultimate = 1, live = 0;
	onode* lives[8];
	for (int i = 0; i < 8; ++i)
	{
		aabb cb = o->bounds;
		if (i & 1) cb.min.x = o->pivot.x; else cb.max.x = o->pivot.x;
		if (i & 2) cb.min.y = o->pivot.y; else cb.max.y = o->pivot.y;
		if (i & 4) cb.min.z = o->pivot.z; else cb.max.z = o->pivot.z;
		onode* c = octree_node(T, o->evaluator, cb, coalesce, depth + 1, max_depth);
		if (c->evaluator == NULL) { onode_destroy(c); o->children[i] = NULL; }
		else
		{
			o->children[i] = c;
			uniform &= node_equal(o->evaluator, c->evaluator);
			penultimate &= c->terminus;
			lives[live++] = c;
		}
	}
	if (live == 0)
	{
		o->evaluator = NULL;
		o->terminus = 1;
		return;
	}
	o->bounds = lives[0]->bounds;
	for (int i = 1; i < live; ++i)
	{
		o->bounds.min = gmin3(o->bounds.min, lives[i]->bounds.min);
		o->bounds.max = gmax3(o->bounds.max, lives[i]->bounds.max);
	}
	int limit = depth > 3 ? depth : 3;
	if (coalesce && ((penultimate && uniform) || o->evaluator_leaves <= limit))
	{
		for (int i = 0; i < 8; ++i) { onode_destroy(o->children[i]); o->children[i] = NULL; }
		o->terminus = 1;
	}
}

tgo_octree* tgo_octree_create(tgo_tree* tree, float target, int coalesce, int max_depth)
{
	if (!node_finite(tree->root)) return NULL;
	aabb b = aabb_bounding_cube(node_bounds(tree->root, 0));
	if (!aabb_degenerate(b)) { b.min = sub3(b.min, V3(0, 0, 0)); b.max = add3(b.max, V3(0, 0, 0)); }
	if (aabb_volume(b) == 0.0f) return NULL;
	tgo_octree* T = (tgo_octree*)calloc(1, sizeof(tgo_octree));
	T->tree = tree;
	T->target = target;
	T->root = octree_node(T, tree->root, b, coalesce, 1, max_depth);
	if (!T->root->evaluator) { tgo_octree_free(T); return NULL; }
	return T;
}

void tgo_octree_free(tgo_octree* T)
{
	if (!T) return;
	onode_destroy(T->root);
	arena_free(&T->mem);
	free(T);
}

/* Descend(Point, Exact=true), sdf_evaluator.cpp:1801-1835. */
static onode* octree_descend(onode* o, v3 p, int exact)
{
	if (!o->terminus)
	{
		int i = 0;
		if (p.x > o->pivot.x) i |= 1;
		if (p.y > o->pivot.y) i |= 2;
		if (p.z > o->pivot.z) i |= 4;
		onode* c = o->children[i];
		if (c)
		{
			onode* f = octree_descend(c, p, exact);
			if (f || !exact) return f;
		}
		else if (!exact) return NULL;
	}
	return o->evaluator ? o : NULL;
}

static float octree_eval_point(tgo_octree* T, v3 p, int exact)
{
	onode* o = octree_descend(T->root, p, exact);
	if (!o) return INFINITY;
	return interp_eval(o->program.w, o->program.n, o->stack_size, p);
}

typedef struct { float* nodes; int32_t* children; uint32_t* words; int n_nodes, cap_nodes, n_words, cap_words; } dumpbuf;

static int dump_node(onode* o, dumpbuf* d)
{
	int idx = d->n_nodes++;
	if (d->n_nodes > d->cap_nodes)
	{
		d->cap_nodes = d->cap_nodes ? d->cap_nodes * 2 : 64;
		d->nodes = (float*)realloc(d->nodes, sizeof(float) * 14 * (size_t)d->cap_nodes);
		d->children = (int32_t*)realloc(d->children, sizeof(int32_t) * 8 * (size_t)d->cap_nodes);
	}
	float* N = d->nodes + (size_t)idx * 14;
	N[0] = o->pivot.x; N[1] = o->pivot.y; N[2] = o->pivot.z;
	N[3] = o->bounds.min.x; N[4] = o->bounds.min.y; N[5] = o->bounds.min.z;
	N[6] = o->bounds.max.x; N[7] = o->bounds.max.y; N[8] = o->bounds.max.z;
	N[9] = o->terminus ? 1.0f : 0.0f;
	N[10] = o->evaluator ? 1.0f : 0.0f;
	N[11] = (float)d->n_words;
	/* A cell whose evaluator Populate dropped keeps no program. */
	const int nwords = o->evaluator ? o->program.n : 0;
	N[12] = (float)nwords;
	N[13] = (float)(o->evaluator ? o->stack_size : 0);
	for (int i = 0; i < 8; ++i) d->children[(size_t)idx * 8 + i] = -1;
	for (int i = 0; i < nwords; ++i)
	{
		if (d->n_words == d->cap_words) { d->cap_words = d->cap_words ? d->cap_words * 2 : 1024; d->words = (uint32_t*)realloc(d->words, 4 * (size_t)d->cap_words); }
		d->words[d->n_words++] = o->program.w[i];
	}
	if (!o->terminus)
	{
		for (int c = 0; c < 8; ++c)
		{
			if (o->children[c])
			{
				int ci = dump_node(o->children[c], d);
				d->children[(size_t)idx * 8 + c] = ci;
			}
		}
	}
	return idx;
}

int tgo_octree_dump(tgo_octree* T, float** nodes, int32_t** children, uint32_t** w, int* wc)
{
	dumpbuf d = { 0 };
	dump_node(T->root, &d);
	*nodes = d.nodes;
	*children = d.children;
	*w = d.words ? d.words : (uint32_t*)malloc(4);
	*wc = d.n_words;
	return d.n_nodes;
}

void tgo_octree_eval(tgo_octree* T, int64_t n, const float* p, int exact, float* o)
{
	for (int64_t i = 0; i < n; ++i) o[i] = octree_eval_point(T, V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]), exact);
}

static node* octree_select(tgo_octree* T, v3 p)
{
	onode* o = octree_descend(T->root, p, 1);
	return o ? o->evaluator : NULL;
}

void tgo_octree_gradient(tgo_octree* T, int64_t n, const float* p, float* o)
{
	for (int64_t i = 0; i < n; ++i)
	{
		v3 q = V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]);
		v3 g = node_gradient(octree_select(T, q), q);
		o[i * 3] = g.x; o[i * 3 + 1] = g.y; o[i * 3 + 2] = g.z;
	}
}

void tgo_octree_color(tgo_octree* T, int64_t n, const float* p, uint8_t* o)
{
	for (int64_t i = 0; i < n; ++i)
	{
		v3 q = V3(p[i * 3], p[i * 3 + 1], p[i * 3 + 2]);
		color_bytes(T->tree, node_material(octree_select(T, q), q), o + i * 3);
	}
}

int tgo_octree_has_paint(tgo_octree* T) { return node_has_paint(T->root->evaluator); }

/* ------------------------------------------------------------------------------------ */
/* Thread helper.                                                                        */
typedef struct
{
	void (*fn)(void* ctx, int64_t item);
	void* ctx;
	int64_t count;
	int64_t chunk;
	atomic_llong next;
} work;

static void* work_thread(void* arg)
{
	work* w = (work*)arg;
	for (;;)
	{
		int64_t s = atomic_fetch_add(&w->next, w->chunk);
		if (s >= w->count) break;
		int64_t e = s + w->chunk < w->count ? s + w->chunk : w->count;
		for (int64_t i = s; i < e; ++i) w->fn(w->ctx, i);
	}
	return NULL;
}

int tgo_hardware_threads(void)
{
	long n = sysconf(_SC_NPROCESSORS_ONLN);
	return n > 0 ? (int)n : 1;
}

static void run_parallel(int threads, int64_t count, int64_t chunk, void (*fn)(void*, int64_t), void* ctx)
{
	if (threads <= 0) threads = tgo_hardware_threads();
	work w;
	w.fn = fn; w.ctx = ctx; w.count = count; w.chunk = chunk < 1 ? 1 : chunk;
	atomic_init(&w.next, 0);
	if (threads == 1) { work_thread(&w); return; }
	pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
	for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, work_thread, &w);
	for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
	free(th);
}

typedef struct { tgo_octree* T; float x0, y0, z0, dx, dy, dz; int64_t nx, ny; float* out; } grid_ctx;

static void grid_slice(void* c, int64_t k)
{
	grid_ctx* g = (grid_ctx*)c;
	float z = g->z0 + (float)k * g->dz;
	for (int64_t j = 0; j < g->ny; ++j)
	{
		float y = g->y0 + (float)j * g->dy;
		for (int64_t i = 0; i < g->nx; ++i)
		{
			float x = g->x0 + (float)i * g->dx;
			g->out[(k * g->ny + j) * g->nx + i] = octree_eval_point(g->T, V3(x, y, z), 1);
		}
	}
}

void tgo_octree_grid(tgo_octree* T, float x0, float y0, float z0, float dx, float dy, float dz,
                     int64_t nx, int64_t ny, int64_t nz, int threads, float* out)
{
	grid_ctx g = { T, x0, y0, z0, dx, dy, dz, nx, ny, out };
	run_parallel(threads, nz, 1, grid_slice, &g);
}

/* ------------------------------------------------------------------------------------ */
/* Naive surface nets (surface_nets.cpp:829-1122).                                       */
typedef struct
{
	tgo_octree* T;
	float gx, gy, gz, dx, dy, dz;
	int64_t sx, sy, sz;
	int faithful;
	float* corners;          /* (sx+1)(sy+1)(sz+1) when !faithful */
	int64_t* cube_vertex;    /* per cell: vertex slot within its slice, or -1 */
	float* slice_vertices;   /* per slice k: dynamic list */
	int64_t* slice_count;
	float** slice_buf;
	int64_t* slice_cap;
	int64_t* slice_cells;    /* per slice: cell indices of the vertices */
	int64_t** slice_cellbuf;
	int64_t* vertex_base;    /* per slice: first global vertex index */
	uint64_t** face_buf;
	int64_t* face_count;
	int64_t* face_cap;
} sn_ctx;

static inline float world(float g0, int64_t i, float d) { return g0 + (float)i * d; }

static inline float sn_corner(sn_ctx* c, int64_t i, int64_t j, int64_t k)
{
	if (!c->faithful) return c->corners[(k * (c->sy + 1) + j) * (c->sx + 1) + i];
	return octree_eval_point(c->T, V3(world(c->gx, i, c->dx), world(c->gy, j, c->dy), world(c->gz, k, c->dz)), 1);
}

static void sn_corner_slice(void* cv, int64_t k)
{
	sn_ctx* c = (sn_ctx*)cv;
	for (int64_t j = 0; j <= c->sy; ++j)
		for (int64_t i = 0; i <= c->sx; ++i)
			c->corners[(k * (c->sy + 1) + j) * (c->sx + 1) + i] =
				octree_eval_point(c->T, V3(world(c->gx, i, c->dx), world(c->gy, j, c->dy), world(c->gz, k, c->dz)), 1);
}

static const int EDGES[12][2] = { {0,1},{1,2},{2,3},{3,0},{4,5},{5,6},{6,7},{7,4},{0,4},{1,5},{2,6},{3,7} };
static const int CORNER_OFS[8][3] = { {0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1} };

/* FirstLoopInnerThunk over one z-slice, surface_nets.cpp:864-974. */
static void sn_cell_slice(void* cv, int64_t k)
{
	sn_ctx* c = (sn_ctx*)cv;
	const float minx = c->gx, miny = c->gy, minz = c->gz;
	const float maxx = c->gx + (float)c->sx * c->dx;
	const float maxy = c->gy + (float)c->sy * c->dy;
	const float maxz = c->gz + (float)c->sz * c->dz;
	for (int64_t j = 0; j < c->sy; ++j)
	{
		for (int64_t i = 0; i < c->sx; ++i)
		{
			float v[8];
			for (int q = 0; q < 8; ++q) v[q] = sn_corner(c, i + CORNER_OFS[q][0], j + CORNER_OFS[q][1], k + CORNER_OFS[q][2]);
			int bip[12], any = 0;
			for (int e = 0; e < 12; ++e)
			{
				bip[e] = (v[EDGES[e][0]] >= 0.0f) != (v[EDGES[e][1]] >= 0.0f);
				any |= bip[e];
			}
			int64_t cell = i + j * c->sx + k * c->sx * c->sy;
			if (!any) { c->cube_vertex[cell] = -1; continue; }
			float sumx = 0.0f, sumy = 0.0f, sumz = 0.0f;
			int count = 0;
			for (int e = 0; e < 12; ++e)
			{
				if (!bip[e]) continue;
				const int* a = CORNER_OFS[EDGES[e][0]];
				const int* b = CORNER_OFS[EDGES[e][1]];
				float p1x = (float)i + (float)a[0], p1y = (float)j + (float)a[1], p1z = (float)k + (float)a[2];
				float p2x = (float)i + (float)b[0], p2y = (float)j + (float)b[1], p2z = (float)k + (float)b[2];
				float s1 = v[EDGES[e][0]], s2 = v[EDGES[e][1]];
				float t = (0.0f - s1) / (s2 - s1);
				sumx = sumx + (p1x + t * (p2x - p1x));
				sumy = sumy + (p1y + t * (p2y - p1y));
				sumz = sumz + (p1z + t * (p2z - p1z));
				++count;
			}
			float nf = (float)count;
			float cx = sumx / nf, cy = sumy / nf, cz = sumz / nf;
			float vx = minx + (maxx - minx) * (cx - 0.0f) / ((float)c->sx - 0.0f);
			float vy = miny + (maxy - miny) * (cy - 0.0f) / ((float)c->sy - 0.0f);
			float vz = minz + (maxz - minz) * (cz - 0.0f) / ((float)c->sz - 0.0f);
			int64_t n = c->slice_count[k];
			if (n == c->slice_cap[k])
			{
				c->slice_cap[k] = c->slice_cap[k] ? c->slice_cap[k] * 2 : 256;
				c->slice_buf[k] = (float*)realloc(c->slice_buf[k], sizeof(float) * 3 * (size_t)c->slice_cap[k]);
				c->slice_cellbuf[k] = (int64_t*)realloc(c->slice_cellbuf[k], sizeof(int64_t) * (size_t)c->slice_cap[k]);
			}
			c->slice_buf[k][n * 3 + 0] = vx;
			c->slice_buf[k][n * 3 + 1] = vy;
			c->slice_buf[k][n * 3 + 2] = vz;
			c->slice_cellbuf[k][n] = cell;
			c->cube_vertex[cell] = n;
			c->slice_count[k] = n + 1;
		}
	}
}

static inline int64_t sn_vertex_of(sn_ctx* c, int64_t i, int64_t j, int64_t k)
{
	int64_t cell = i + j * c->sx + k * c->sx * c->sy;
	int64_t local = c->cube_vertex[cell];
	return local < 0 ? -1 : c->vertex_base[k] + local;
}

/* SecondLoopThunk over the active cells of one z-slice, surface_nets.cpp:1001-1121. */
static void sn_face_slice(void* cv, int64_t k)
{
	sn_ctx* c = (sn_ctx*)cv;
	if (k == 0) return;
	for (int64_t n = 0; n < c->slice_count[k]; ++n)
	{
		int64_t cell = c->slice_cellbuf[k][n];
		int64_t i = cell % c->sx;
		int64_t j = (cell / c->sx) % c->sy;
		if (i == 0 || j == 0) continue;
		int64_t v0 = c->vertex_base[k] + n;
		int64_t nb[6][3] = { {i - 1, j, k}, {i - 1, j - 1, k}, {i, j - 1, k}, {i, j - 1, k - 1}, {i, j, k - 1}, {i - 1, j, k - 1} };
		/* edge scalars (0,4), (3,0), (0,1): six evaluations, as the reference makes */
		float es[3][2] = {
			{ sn_corner(c, i, j, k), sn_corner(c, i, j, k + 1) },
			{ sn_corner(c, i, j + 1, k), sn_corner(c, i, j, k) },
			{ sn_corner(c, i, j, k), sn_corner(c, i + 1, j, k) } };
		static const int quad[3][3] = { {0, 1, 2}, {0, 5, 4}, {2, 3, 4} };
		for (int q = 0; q < 3; ++q)
		{
			int64_t nv[3];
			int ok = 1;
			for (int m = 0; m < 3; ++m)
			{
				const int64_t* g = nb[quad[q][m]];
				nv[m] = sn_vertex_of(c, g[0], g[1], g[2]);
				if (nv[m] < 0) ok = 0;
			}
			if (!ok) continue;
			int64_t v1, v2, v3;
			if (es[q][1] > es[q][0]) { v1 = nv[0]; v2 = nv[1]; v3 = nv[2]; }
			else { v1 = nv[2]; v2 = nv[1]; v3 = nv[0]; }
			int64_t f = c->face_count[k];
			if (f + 2 > c->face_cap[k])
			{
				c->face_cap[k] = c->face_cap[k] ? c->face_cap[k] * 2 : 512;
				c->face_buf[k] = (uint64_t*)realloc(c->face_buf[k], sizeof(uint64_t) * 3 * (size_t)c->face_cap[k]);
			}
			uint64_t* F = c->face_buf[k] + f * 3;
			F[0] = (uint64_t)v0; F[1] = (uint64_t)v1; F[2] = (uint64_t)v2;
			F[3] = (uint64_t)v0; F[4] = (uint64_t)v2; F[5] = (uint64_t)v3;
			c->face_count[k] = f + 2;
		}
	}
}

static double now_seconds(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int64_t tgo_surface_nets(tgo_octree* T, float x0, float y0, float z0, float dx, float dy, float dz,
                         int64_t sx, int64_t sy, int64_t sz, int threads, int faithful,
                         float** vertices, uint64_t** cubes, uint64_t** faces, int64_t* face_count, double* seconds)
{
	/* The reference's FirstLoopThunk swaps loop variables when one axis is strictly the
	 * longest (surface_nets.cpp:976-999); only grids without a strictly longest axis are
	 * restated here. */
	int xl = sx > sy && sx > sz, yl = sy > sx && sy > sz;
	if (xl || yl) return -1;
	double t0 = now_seconds();
	sn_ctx c;
	memset(&c, 0, sizeof c);
	c.T = T; c.gx = x0; c.gy = y0; c.gz = z0; c.dx = dx; c.dy = dy; c.dz = dz; c.sx = sx; c.sy = sy; c.sz = sz;
	c.faithful = faithful;
	if (!faithful)
	{
		c.corners = (float*)malloc(sizeof(float) * (size_t)((sx + 1) * (sy + 1) * (sz + 1)));
		run_parallel(threads, sz + 1, 1, sn_corner_slice, &c);
	}
	c.cube_vertex = (int64_t*)malloc(sizeof(int64_t) * (size_t)(sx * sy * sz));
	c.slice_count = (int64_t*)calloc((size_t)sz, sizeof(int64_t));
	c.slice_cap = (int64_t*)calloc((size_t)sz, sizeof(int64_t));
	c.slice_buf = (float**)calloc((size_t)sz, sizeof(float*));
	c.slice_cellbuf = (int64_t**)calloc((size_t)sz, sizeof(int64_t*));
	c.vertex_base = (int64_t*)calloc((size_t)sz + 1, sizeof(int64_t));
	c.face_buf = (uint64_t**)calloc((size_t)sz, sizeof(uint64_t*));
	c.face_count = (int64_t*)calloc((size_t)sz, sizeof(int64_t));
	c.face_cap = (int64_t*)calloc((size_t)sz, sizeof(int64_t));
	run_parallel(threads, sz, 1, sn_cell_slice, &c);
	for (int64_t k = 0; k < sz; ++k) c.vertex_base[k + 1] = c.vertex_base[k] + c.slice_count[k];
	run_parallel(threads, sz, 1, sn_face_slice, &c);
	*seconds = now_seconds() - t0;

	int64_t nv = c.vertex_base[sz];
	int64_t nf = 0;
	for (int64_t k = 0; k < sz; ++k) nf += c.face_count[k];
	float* V = (float*)malloc(sizeof(float) * 3 * (size_t)(nv ? nv : 1));
	uint64_t* C = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(nv ? nv : 1));
	uint64_t* F = (uint64_t*)malloc(sizeof(uint64_t) * 3 * (size_t)(nf ? nf : 1));
	int64_t fo = 0;
	for (int64_t k = 0; k < sz; ++k)
	{
		int64_t b = c.vertex_base[k];
		if (c.slice_count[k])
		{
			memcpy(V + b * 3, c.slice_buf[k], sizeof(float) * 3 * (size_t)c.slice_count[k]);
			for (int64_t n = 0; n < c.slice_count[k]; ++n) C[b + n] = (uint64_t)c.slice_cellbuf[k][n];
		}
		if (c.face_count[k]) memcpy(F + fo * 3, c.face_buf[k], sizeof(uint64_t) * 3 * (size_t)c.face_count[k]);
		fo += c.face_count[k];
		free(c.slice_buf[k]); free(c.slice_cellbuf[k]); free(c.face_buf[k]);
	}
	free(c.corners); free(c.cube_vertex); free(c.slice_count); free(c.slice_cap); free(c.slice_buf);
	free(c.slice_cellbuf); free(c.vertex_base); free(c.face_buf); free(c.face_count); free(c.face_cap);
	*vertices = V; *cubes = C; *faces = F; *face_count = nf;
	return nv;
}

typedef struct { tgo_octree* T; const float* v; float* normals; uint8_t* colors; int paint; } attr_ctx;

static void attr_one(void* cv, int64_t i)
{
	attr_ctx* a = (attr_ctx*)cv;
	v3 q = V3(a->v[i * 3], a->v[i * 3 + 1], a->v[i * 3 + 2]);
	node* e = octree_select(a->T, q);
	v3 g = node_gradient(e, q);
	a->normals[i * 3] = g.x; a->normals[i * 3 + 1] = g.y; a->normals[i * 3 + 2] = g.z;
	if (a->colors) color_bytes(a->T->tree, node_material(e, q), a->colors + i * 3);
}

void tgo_vertex_attributes(tgo_octree* T, int64_t n, const float* v, int threads, float* normals, uint8_t* colors)
{
	attr_ctx a = { T, v, normals, colors, 1 };
	run_parallel(threads, n, 256, attr_one, &a);
}

/* ------------------------------------------------------------------------------------ */
/* SDFNode::RayMarch, sdf_evaluator.cpp:336-353.                                          */
typedef struct { tgo_tree* t; const float* o; const float* d; int iters; float eps; uint8_t* hit; float* travel; float* pos; } ray_ctx;

static void ray_one(void* cv, int64_t r)
{
	ray_ctx* c = (ray_ctx*)cv;
	v3 start = V3(c->o[r * 3], c->o[r * 3 + 1], c->o[r * 3 + 2]);
	v3 dir = normalize3(V3(c->d[r * 3], c->d[r * 3 + 1], c->d[r * 3 + 2]));
	v3 pos = start;
	float travel = 0.0f;
	int hit = 0;
	for (int i = 0; i < c->iters; ++i)
	{
		float dist = node_eval(c->t->root, pos);
		if (dist <= c->eps) { hit = 1; break; }
		travel = travel + dist;
		pos = add3(muls3(dir, travel), start);
	}
	if (!hit) travel = INFINITY;
	c->hit[r] = (uint8_t)hit;
	c->travel[r] = travel;
	c->pos[r * 3] = pos.x; c->pos[r * 3 + 1] = pos.y; c->pos[r * 3 + 2] = pos.z;
}

/* Lua's magnet cast (mode 1: dir = normalize(target - origin)) and SDFModel::RayMarch (mode
 * 2: the ray taken into the model frame {quat w x y z, translation, scale}, 1000 iterations,
 * epsilon 0.001), serially (lua_sdf.cpp:410-437, sdf_model.cpp:261-266). */
void tgo_ray_query(tgo_tree* t, int mode, const float* frame, int64_t n, const float* o, const float* d, int iters, float eps,
                   uint8_t* hit, float* travel, float* pos)
{
	xform X = xf_identity();
	if (mode == 2)
	{
		X.rot.w = frame[0]; X.rot.x = frame[1]; X.rot.y = frame[2]; X.rot.z = frame[3];
		X.trans = V3(frame[4], frame[5], frame[6]);
		X.scale = frame[7];
	}
	for (int64_t r = 0; r < n; ++r)
	{
		v3 origin = V3(o[r * 3], o[r * 3 + 1], o[r * 3 + 2]);
		v3 dir = V3(d[r * 3], d[r * 3 + 1], d[r * 3 + 2]);
		int it = iters;
		float e = eps;
		if (mode == 1) dir = normalize3(sub3(dir, origin));
		else
		{
			origin = xf_apply_inv(&X, origin);
			dir = qrot(qinv(X.rot), dir);
			it = 1000;
			e = 0.001f;
		}
		float rd[3] = { dir.x, dir.y, dir.z }, ro[3] = { origin.x, origin.y, origin.z };
		ray_ctx c = { t, ro, rd, it, e, hit + r, travel + r, pos + r * 3 };
		ray_one(&c, 0);
	}
}

void tgo_raymarch(tgo_tree* t, int64_t n, const float* o, const float* d, int iters, float eps, int threads,
                  uint8_t* hit, float* travel, float* pos)
{
	ray_ctx c = { t, o, d, iters, eps, hit, travel, pos };
	run_parallel(threads, n, 64, ray_one, &c);
}

/* ------------------------------------------------------------------------------------ */
/* Sodapop's meshing chain, MeshingJob::NaiveSurfaceNets (sodapop.cpp:562-897), serially.  */

typedef struct { onode** items; int n, cap; } leaf_list;

/* SDFOctree::LinkLeaves (sdf_evaluator.cpp:1912-1947): the terminus cells with an
 * evaluator. */
static void collect_leaves(onode* o, leaf_list* out)
{
	if (!o) return;
	if (o->terminus)
	{
		if (!o->evaluator) return;
		if (out->n == out->cap)
		{
			out->cap = out->cap ? out->cap * 2 : 256;
			out->items = (onode**)realloc(out->items, sizeof(onode*) * (size_t)out->cap);
		}
		out->items[out->n++] = o;
		return;
	}
	for (int i = 0; i < 8; ++i) collect_leaves(o->children[i], out);
}

/* SDFOctree::Walk with the incomplete search (sodapop.cpp:108-124), each found cell
 * populated right away (the cells are disjoint, so the order does not matter). */
static void populate_incomplete(tgo_octree* T, onode* o)
{
	if (!o) return;
	if (o->terminus || o->incomplete)
	{
		if (o->incomplete)
		{
			octree_populate(T, o, 0, 3, -1);
		}
		return;
	}
	for (int i = 0; i < 8; ++i) populate_incomplete(T, o->children[i]);
}

static inline float sp_implicit(tgo_octree* T, float x, float y, float z)
{
	/* glm::clamp(Eval(p, false), -100, 100): min(max(x, lo), hi) with glm's comparisons. */
	return gclamp(octree_eval_point(T, V3(x, y, z), 0), -100.0f, 100.0f);
}

/* MaterialPBRBR::Eval(P, N, V) with V = N (material.cpp:33-40): SampleColor x BSDF. */
static v3 pbrbr(const float* rgb, v3 n)
{
	float dd = gmax(dot3(n, normalize3(add3(muls3(n, 0.75f), n))), 0.0f);
	float D = powf(dd, 2.0f);
	float F = 1.0f - gmax(dot3(n, n), 0.0f);
	float bsdf = D + F * 0.25f;
	return V3(rgb[0] * bsdf, rgb[1] * bsdf, rgb[2] * bsdf);
}

tgo_octree* tgo_meshing_octree_create(tgo_tree* tree)
{
	tgo_octree* T = tgo_octree_create(tree, 0.25f, 0, 3);
	if (T) populate_incomplete(T, T->root);
	return T;
}

int64_t tgo_sodapop(tgo_tree* tree, float density, float** positions, float** normals, float** colors, uint64_t** faces,
	int64_t* face_count, float* grid_out)
{
	/* SDFOctree::Create(.25, false, 3), then every incomplete cell populated on its own with
	 * Populate(false, 3, -1) (sodapop.cpp:565-567): the incomplete cells' ancestors keep the
	 * bounds they took at depth 3. */
	tgo_octree* T = tgo_octree_create(tree, 0.25f, 0, 3);
	if (!T) return -1;
	populate_incomplete(T, T->root);

	/* NaiveSurfaceNetsScratch (sodapop.cpp:150-177). */
	const aabb B = T->root->bounds;
	const v3 ext = sub3(B.max, B.min);
	const float fl = floorf(density);
	const v3 spu = gmax3(mul3(ext, V3(fl, fl, fl)), V3(8.0f, 8.0f, 8.0f));
	int64_t sx = (int64_t)ceilf(spu.x), sy = (int64_t)ceilf(spu.y), sz = (int64_t)ceilf(spu.z);
	const float dx = ext.x / (float)sx, dy = ext.y / (float)sy, dz = ext.z / (float)sz;
	const float gx = B.min.x - dx * 2.0f, gy = B.min.y - dy * 2.0f, gz = B.min.z - dz * 2.0f;
	sx += 3; sy += 3; sz += 3;
	grid_out[0] = gx; grid_out[1] = gy; grid_out[2] = gz;
	grid_out[3] = dx; grid_out[4] = dy; grid_out[5] = dz;
	grid_out[6] = (float)sx; grid_out[7] = (float)sy; grid_out[8] = (float)sz;

	/* Point cache: every grid index inside a leaf's aligned box whose 64-entry bucket
	 * exists (sodapop.cpp:613-644), in increasing order (std::set per bucket). */
	const int64_t range = sx * sy * sz;
	const int64_t bucket = range < 64 ? range : 64;
	const int64_t limit = ((range + bucket - 1) / bucket) * bucket;
	uint8_t* cached = (uint8_t*)calloc((size_t)limit, 1);
	leaf_list leaves = { NULL, 0, 0 };
	collect_leaves(T->root, &leaves);
	for (int l = 0; l < leaves.n; ++l)
	{
		const onode* o = leaves.items[l];
		const float amnx = floorf(gmax(0.0f, o->bounds.min.x - gx) / dx);
		const float amny = floorf(gmax(0.0f, o->bounds.min.y - gy) / dy);
		const float amnz = floorf(gmax(0.0f, o->bounds.min.z - gz) / dz);
		const float amxx = ceilf((o->bounds.max.x - gx) / dx);
		const float amxy = ceilf((o->bounds.max.y - gy) / dy);
		const float amxz = ceilf((o->bounds.max.z - gz) / dz);
		for (float z = amnz; z <= amxz; ++z)
			for (float y = amny; y <= amxy; ++y)
				for (float x = amnx; x <= amxx; ++x)
				{
					const int64_t index = (int64_t)x + (int64_t)y * sx + (int64_t)z * sx * sy;
					if (index < limit) cached[index] = 1;
				}
	}
	free(leaves.items);

	/* FirstLoopInnerThunk per cached point (surface_nets.cpp:864-974). */
	const float maxx = gx + (float)sx * dx, maxy = gy + (float)sy * dy, maxz = gz + (float)sz * dz;
	int64_t* cube_vertex = (int64_t*)malloc(sizeof(int64_t) * (size_t)limit);
	int64_t nv = 0, capv = 1024;
	float* V = (float*)malloc(sizeof(float) * 3 * (size_t)capv);
	int64_t* VC = (int64_t*)malloc(sizeof(int64_t) * (size_t)capv);
	for (int64_t index = 0; index < limit; ++index)
	{
		cube_vertex[index] = -1;
		if (!cached[index]) continue;
		const int64_t i = index % sx, j = (index / sx) % sy, k = index / (sx * sy);
		float v[8];
		for (int q = 0; q < 8; ++q)
			v[q] = sp_implicit(T, world(gx, i + CORNER_OFS[q][0], dx), world(gy, j + CORNER_OFS[q][1], dy),
				world(gz, k + CORNER_OFS[q][2], dz));
		float sumx = 0.0f, sumy = 0.0f, sumz = 0.0f;
		int count = 0;
		for (int e = 0; e < 12; ++e)
		{
			const float s1 = v[EDGES[e][0]], s2 = v[EDGES[e][1]];
			if ((s1 >= 0.0f) == (s2 >= 0.0f)) continue;
			const int* a = CORNER_OFS[EDGES[e][0]];
			const int* b = CORNER_OFS[EDGES[e][1]];
			float p1x = (float)i + (float)a[0], p1y = (float)j + (float)a[1], p1z = (float)k + (float)a[2];
			float p2x = (float)i + (float)b[0], p2y = (float)j + (float)b[1], p2z = (float)k + (float)b[2];
			float t = (0.0f - s1) / (s2 - s1);
			sumx = sumx + (p1x + t * (p2x - p1x));
			sumy = sumy + (p1y + t * (p2y - p1y));
			sumz = sumz + (p1z + t * (p2z - p1z));
			++count;
		}
		if (!count) continue;
		float nf = (float)count;
		float cx = sumx / nf, cy = sumy / nf, cz = sumz / nf;
		if (nv == capv)
		{
			capv *= 2;
			V = (float*)realloc(V, sizeof(float) * 3 * (size_t)capv);
			VC = (int64_t*)realloc(VC, sizeof(int64_t) * (size_t)capv);
		}
		V[nv * 3 + 0] = gx + (maxx - gx) * (cx - 0.0f) / ((float)sx - 0.0f);
		V[nv * 3 + 1] = gy + (maxy - gy) * (cy - 0.0f) / ((float)sy - 0.0f);
		V[nv * 3 + 2] = gz + (maxz - gz) * (cz - 0.0f) / ((float)sz - 0.0f);
		VC[nv] = index;
		cube_vertex[index] = nv++;
	}

	/* SecondLoopThunk per vertex (surface_nets.cpp:1001-1121). */
	int64_t nf = 0, capf = 1024;
	uint64_t* F = (uint64_t*)malloc(sizeof(uint64_t) * 3 * (size_t)capf);
	for (int64_t n = 0; n < nv; ++n)
	{
		const int64_t cell = VC[n];
		const int64_t i = cell % sx, j = (cell / sx) % sy, k = cell / (sx * sy);
		if (i == 0 || j == 0 || k == 0) continue;
		const int64_t nb[6] = { cell - 1, cell - 1 - sx, cell - sx, cell - sx - sx * sy, cell - sx * sy, cell - 1 - sx * sy };
		const float c0 = sp_implicit(T, world(gx, i, dx), world(gy, j, dy), world(gz, k, dz));
		const float es[3][2] = {
			{ c0, sp_implicit(T, world(gx, i, dx), world(gy, j, dy), world(gz, k + 1, dz)) },
			{ sp_implicit(T, world(gx, i, dx), world(gy, j + 1, dy), world(gz, k, dz)), c0 },
			{ c0, sp_implicit(T, world(gx, i + 1, dx), world(gy, j, dy), world(gz, k, dz)) } };
		static const int quad[3][3] = { {0, 1, 2}, {0, 5, 4}, {2, 3, 4} };
		for (int q = 0; q < 3; ++q)
		{
			int64_t w[3];
			int ok = 1;
			for (int m = 0; m < 3; ++m)
			{
				const int64_t c = nb[quad[q][m]];
				w[m] = (c >= 0 && c < limit) ? cube_vertex[c] : -1;
				if (w[m] < 0) ok = 0;
			}
			if (!ok) continue;
			int64_t v1, v2, v3;
			if (es[q][1] > es[q][0]) { v1 = w[0]; v2 = w[1]; v3 = w[2]; }
			else { v1 = w[2]; v2 = w[1]; v3 = w[0]; }
			if (nf + 2 > capf)
			{
				capf *= 2;
				F = (uint64_t*)realloc(F, sizeof(uint64_t) * 3 * (size_t)capf);
			}
			uint64_t* f = F + nf * 3;
			f[0] = (uint64_t)n; f[1] = (uint64_t)v1; f[2] = (uint64_t)v2;
			f[3] = (uint64_t)n; f[4] = (uint64_t)v2; f[5] = (uint64_t)v3;
			nf += 2;
		}
	}

	/* Gradient normals and material colours (sodapop.cpp:815-872). */
	float* N = (float*)malloc(sizeof(float) * 3 * (size_t)(nv ? nv : 1));
	float* C4 = (float*)malloc(sizeof(float) * 4 * (size_t)(nv ? nv : 1));
	static const float white[3] = { 1.0f, 1.0f, 1.0f };
	for (int64_t n = 0; n < nv; ++n)
	{
		const v3 q = V3(V[n * 3], V[n * 3 + 1], V[n * 3 + 2]);
		const node* e = octree_select(T, q);
		const v3 g = node_gradient(e, q);
		N[n * 3] = g.x; N[n * 3 + 1] = g.y; N[n * 3 + 2] = g.z;
		const int mat = node_material(e, q);
		const v3 c = pbrbr(mat >= 0 ? T->tree->materials[mat].rgb : white, g);
		C4[n * 4] = c.x; C4[n * 4 + 1] = c.y; C4[n * 4 + 2] = c.z; C4[n * 4 + 3] = 1.0f;
	}
	free(cached);
	free(cube_vertex);
	free(VC);
	tgo_octree_free(T);
	*positions = V;
	*normals = N;
	*colors = C4;
	*faces = F;
	*face_count = nf;
	return nv;
}

/* ------------------------------------------------------------------------------------ */
/* PointCloudExportThread (export.cpp:384-480), serially in cell order.                   */
int64_t tgo_point_cloud(tgo_octree* T, const float* lo, const float* hi, const float* step, int refine,
	float** points, int32_t** cells)
{
	/* Half = Step / vec3(2.0); Diagonal = length(Half) */
	const v3 Step = V3(step[0], step[1], step[2]);
	const v3 Half = V3(Step.x / 2.0f, Step.y / 2.0f, Step.z / 2.0f);
	const float diag = len3(Half);
	const v3 Start = V3(lo[0], lo[1], lo[2]);
	/* ivec3(ceil((Stop - Start) / Step)) */
	const int ix = (int)ceilf((hi[0] - Start.x) / Step.x);
	const int iy = (int)ceilf((hi[1] - Start.y) / Step.y);
	const int iz = (int)ceilf((hi[2] - Start.z) / Step.z);
	const int slice = ix * iy;
	const int total = ix * iy * iz;
	int64_t n = 0, cap = 1024;
	float* P = (float*)malloc(sizeof(float) * 3 * (size_t)cap);
	int32_t* I = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
	for (int i = 0; i < total; ++i)
	{
		const float Z = (float)(i / slice) * Step.z + Start.z;
		const float Y = (float)((i % slice) / ix) * Step.y + Start.y;
		const float X = (float)(i % ix) * Step.x + Start.x;
		const v3 c = add3(V3(X, Y, Z), Half);
		const float d = octree_eval_point(T, c, 1);
		if (!(fabsf(d) < diag)) continue;
		if (n == cap)
		{
			cap *= 2;
			P = (float*)realloc(P, sizeof(float) * 3 * (size_t)cap);
			I = (int32_t*)realloc(I, sizeof(int32_t) * (size_t)cap);
		}
		P[n * 3] = c.x; P[n * 3 + 1] = c.y; P[n * 3 + 2] = c.z;
		I[n++] = i;
	}
	for (int64_t k = 0; k < n && refine > 0; ++k)
	{
		const v3 V = V3(P[k * 3], P[k * 3 + 1], P[k * 3 + 2]);
		const v3 low = sub3(V, Half), high = add3(V, Half);
		v3 cur = V;
		for (int r = 0; r < refine; ++r)
		{
			const v3 dir = node_gradient(octree_select(T, cur), cur);
			/* Octree->Eval(Cursor) * -1.0 in double, stored to float: the exact negation. */
			const float dist = (float)((double)octree_eval_point(T, cur, 1) * -1.0);
			cur = add3(cur, muls3(dir, dist));
		}
		/* glm::clamp(x, lo, hi) = min(max(x, lo), hi) per component */
		cur = gmin3(gmax3(cur, low), high);
		if (len3(sub3(V, cur)) <= diag)
		{
			P[k * 3] = cur.x; P[k * 3 + 1] = cur.y; P[k * 3 + 2] = cur.z;
		}
	}
	*points = P;
	*cells = I;
	return n;
}

/* ------------------------------------------------------------------------------------ */
/* VoxExport's voxel test (magica.cpp:27-69), serially in cell order: the voxels whose     */
/* centre's full-tree distance is within the half-voxel radius.                            */
static v3 glm_mix3(v3 x, v3 y, v3 a)
{
	/* glm::mix(x, y, a) for vectors: x * (1 - a) + y * a */
	const v3 one_minus = V3(1.0f - a.x, 1.0f - a.y, 1.0f - a.z);
	return add3(mul3(x, one_minus), mul3(y, a));
}

int64_t tgo_vox(tgo_tree* tree, float grid_size, int color_index, int32_t* size_out, float* radius_out, int32_t** voxels)
{
	const aabb B = node_bounds(tree->root, 0);
	/* ivec3(glm::ceil(Max - Min) * GridSize) */
	const int sx = (int)(ceilf(B.max.x - B.min.x) * grid_size);
	const int sy = (int)(ceilf(B.max.y - B.min.y) * grid_size);
	const int sz = (int)(ceilf(B.max.z - B.min.z) * grid_size);
	const v3 fs = V3((float)sx, (float)sy, (float)sz);
	const v3 a0 = V3(0.5f / fs.x, 0.5f / fs.y, 0.5f / fs.z);
	/* glm::distance(Min, mix(Min, Max, Alpha)) = length(mix - Min) */
	const float radius = len3(sub3(glm_mix3(B.min, B.max, a0), B.min));
	const int slice = sx * sy;
	const int total = sx * sy * sz;
	const int color = abs(color_index) % 255 + 1;
	int64_t n = 0, cap = 1024;
	int32_t* out = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)cap);
	for (int i = 0; i < total; ++i)
	{
		const int z = i / slice, y = (i % slice) / sx, x = i % sx;
		/* vec3(x + .5, ...) converts the double sums to float */
		const v3 alpha = V3((float)((double)x + .5) / fs.x, (float)((double)y + .5) / fs.y, (float)((double)z + .5) / fs.z);
		const v3 p = glm_mix3(B.min, B.max, alpha);
		const float d = node_eval(tree->root, p);
		if (!(fabsf(d) <= radius)) continue;
		if (n == cap)
		{
			cap *= 2;
			out = (int32_t*)realloc(out, sizeof(int32_t) * 4 * (size_t)cap);
		}
		out[n * 4] = x; out[n * 4 + 1] = y; out[n * 4 + 2] = z; out[n * 4 + 3] = color;
		++n;
	}
	size_out[0] = sx; size_out[1] = sy; size_out[2] = sz;
	*radius_out = radius;
	*voxels = out;
	return n;
}
