// Float vector / quaternion / matrix arithmetic for the host side of the export path.
//
// Tangerine does its math with glm 0.9.9.8 (packed, no SIMD paths).  The octree's clip
// decisions and the program words have to come out bit-identical to the reference, so
// every helper here keeps glm's operand order; this file is compiled with
// -ffp-contract=off so that no multiply-add is fused on either x86-64 or Arm.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define TG_HD __host__ __device__ __forceinline__
#else
#define TG_HD inline
#endif

namespace tg
{
	struct Vec3
	{
		float x, y, z;
		TG_HD Vec3() {}
		TG_HD Vec3(float X, float Y, float Z) : x(X), y(Y), z(Z) {}
		TG_HD explicit Vec3(float S) : x(S), y(S), z(S) {}
		TG_HD float& operator[](int i) { return (&x)[i]; }
		TG_HD float operator[](int i) const { return (&x)[i]; }
	};

	TG_HD Vec3 operator+(Vec3 a, Vec3 b) { return { a.x + b.x, a.y + b.y, a.z + b.z }; }
	TG_HD Vec3 operator-(Vec3 a, Vec3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
	TG_HD Vec3 operator*(Vec3 a, Vec3 b) { return { a.x * b.x, a.y * b.y, a.z * b.z }; }
	TG_HD Vec3 operator*(Vec3 a, float s) { return { a.x * s, a.y * s, a.z * s }; }
	TG_HD Vec3 operator/(Vec3 a, float s) { return { a.x / s, a.y / s, a.z / s }; }
	TG_HD bool operator==(Vec3 a, Vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

	// glm::min / glm::max on scalars are ternaries; the reference's own scalar min/max
	// (glm_common.h) are fminf / fmaxf.  Both are needed.
	TG_HD float TernaryMax(float a, float b) { return (a < b) ? b : a; }
	TG_HD float TernaryMin(float a, float b) { return (b < a) ? b : a; }
	TG_HD Vec3 TernaryMax(Vec3 a, Vec3 b) { return { TernaryMax(a.x, b.x), TernaryMax(a.y, b.y), TernaryMax(a.z, b.z) }; }
	TG_HD Vec3 TernaryMin(Vec3 a, Vec3 b) { return { TernaryMin(a.x, b.x), TernaryMin(a.y, b.y), TernaryMin(a.z, b.z) }; }
	TG_HD Vec3 Abs(Vec3 a) { return { fabsf(a.x), fabsf(a.y), fabsf(a.z) }; }
	TG_HD float Dot(Vec3 a, Vec3 b) { Vec3 t = a * b; return t.x + t.y + t.z; }
	TG_HD float Length(Vec3 a) { return sqrtf(Dot(a, a)); }
	TG_HD Vec3 Cross(Vec3 a, Vec3 b)
	{
		return { a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y };
	}
	TG_HD Vec3 Normalize(Vec3 v) { const float s = 1.0f / sqrtf(Dot(v, v)); return v * s; }

	struct Quat
	{
		float w = 1.0f, x = 0.0f, y = 0.0f, z = 0.0f;
		TG_HD bool IsIdentity() const { return w == 1.0f && x == 0.0f && y == 0.0f && z == 0.0f; }
		TG_HD bool operator==(const Quat& o) const { return w == o.w && x == o.x && y == o.y && z == o.z; }
	};

	// q * v (rotation): v + ((cross(q.xyz, v) * w) + cross(q.xyz, cross(q.xyz, v))) * 2
	TG_HD Vec3 Rotate(Quat q, Vec3 v)
	{
		const Vec3 qv(q.x, q.y, q.z);
		const Vec3 uv = Cross(qv, v);
		const Vec3 uuv = Cross(qv, uv);
		return v + ((uv * q.w) + uuv) * 2.0f;
	}

	// Hamilton product p * q.
	TG_HD Quat Mul(Quat p, Quat q)
	{
		Quat r;
		r.w = p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z;
		r.x = p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y;
		r.y = p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z;
		r.z = p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x;
		return r;
	}

	// conjugate(q) / ((w*w + x*x) + (y*y + z*z))
	TG_HD Quat Inverse(Quat q)
	{
		const float d = (q.w * q.w + q.x * q.x) + (q.y * q.y + q.z * q.z);
		return { q.w / d, -q.x / d, -q.y / d, -q.z / d };
	}

	// Column-major 4x4, m[c * 4 + r].
	struct Mat4
	{
		float m[16];
		static Mat4 Identity()
		{
			Mat4 r;
			std::memset(r.m, 0, sizeof r.m);
			r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
			return r;
		}
		float& at(int c, int r) { return m[c * 4 + r]; }
		float at(int c, int r) const { return m[c * 4 + r]; }
	};

	Mat4 MatMul(const Mat4& a, const Mat4& b);
	Mat4 MatFromQuat(Quat q);
	Mat4 MatInverse(const Mat4& m);

	struct AABB
	{
		Vec3 Min, Max;
		bool Degenerate() const;
		AABB BoundingCube() const;
		float Volume() const;
	};

	// Translation / rotation / uniform scale, applied to points as R(p * s) + t.
	struct Transform
	{
		Quat Rotation;
		Vec3 Translation = Vec3(0.0f);
		float Scalation = 1.0f;

		void Move(Vec3 by) { Translation = Translation + by; }
		void Rotate(Quat by) { Translation = tg::Rotate(by, Translation); Rotation = Mul(by, Rotation); }
		void Scale(float by) { Translation = Translation * by; Scalation = Scalation * by; }
		TG_HD Vec3 Apply(Vec3 p) const { return tg::Rotate(Rotation, p * Scalation) + Translation; }
		TG_HD Vec3 ApplyInv(Vec3 p) const { return tg::Rotate(Inverse(Rotation), p - Translation) / Scalation; }
		Mat4 ToMatrix() const;
		AABB ApplyBounds(const AABB& in) const;
		bool operator==(const Transform& o) const
		{
			return Rotation == o.Rotation && Translation == o.Translation && Scalation == o.Scalation;
		}
	};

	inline uint32_t FloatBits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
	inline float BitsFloat(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
}
