// Host float math with glm 0.9.9.8's operand order (see tg_math.hpp).
#include "tg_math.hpp"

#include <cmath>

namespace tg
{
	// Result[c] = ((A[0]*B[c][0] + A[1]*B[c][1]) + A[2]*B[c][2]) + A[3]*B[c][3]
	Mat4 MatMul(const Mat4& a, const Mat4& b)
	{
		Mat4 r;
		for (int c = 0; c < 4; ++c)
		{
			for (int i = 0; i < 4; ++i)
			{
				float t = a.at(0, i) * b.at(c, 0);
				t = t + a.at(1, i) * b.at(c, 1);
				t = t + a.at(2, i) * b.at(c, 2);
				t = t + a.at(3, i) * b.at(c, 3);
				r.at(c, i) = t;
			}
		}
		return r;
	}

	// Rotation matrix of a unit quaternion (the usual 1 - 2(yy + zz) ... form).
	Mat4 MatFromQuat(Quat q)
	{
		Mat4 r = Mat4::Identity();
		const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
		const float xz = q.x * q.z, xy = q.x * q.y, yz = q.y * q.z;
		const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
		r.at(0, 0) = 1.0f - 2.0f * (yy + zz);
		r.at(0, 1) = 2.0f * (xy + wz);
		r.at(0, 2) = 2.0f * (xz - wy);
		r.at(1, 0) = 2.0f * (xy - wz);
		r.at(1, 1) = 1.0f - 2.0f * (xx + zz);
		r.at(1, 2) = 2.0f * (yz + wx);
		r.at(2, 0) = 2.0f * (xz + wy);
		r.at(2, 1) = 2.0f * (yz - wx);
		r.at(2, 2) = 1.0f - 2.0f * (xx + yy);
		return r;
	}

	// General inverse by 2x2 sub-determinants (cofactors) of the lower rows, then
	// division by the determinant taken along the first column.
	Mat4 MatInverse(const Mat4& M)
	{
		auto e = [&](int c, int r) { return M.at(c, r); };
		const float s00 = e(2,2) * e(3,3) - e(3,2) * e(2,3);
		const float s02 = e(1,2) * e(3,3) - e(3,2) * e(1,3);
		const float s03 = e(1,2) * e(2,3) - e(2,2) * e(1,3);
		const float s04 = e(2,1) * e(3,3) - e(3,1) * e(2,3);
		const float s06 = e(1,1) * e(3,3) - e(3,1) * e(1,3);
		const float s07 = e(1,1) * e(2,3) - e(2,1) * e(1,3);
		const float s08 = e(2,1) * e(3,2) - e(3,1) * e(2,2);
		const float s10 = e(1,1) * e(3,2) - e(3,1) * e(1,2);
		const float s11 = e(1,1) * e(2,2) - e(2,1) * e(1,2);
		const float s12 = e(2,0) * e(3,3) - e(3,0) * e(2,3);
		const float s14 = e(1,0) * e(3,3) - e(3,0) * e(1,3);
		const float s15 = e(1,0) * e(2,3) - e(2,0) * e(1,3);
		const float s16 = e(2,0) * e(3,2) - e(3,0) * e(2,2);
		const float s18 = e(1,0) * e(3,2) - e(3,0) * e(1,2);
		const float s19 = e(1,0) * e(2,2) - e(2,0) * e(1,2);
		const float s20 = e(2,0) * e(3,1) - e(3,0) * e(2,1);
		const float s22 = e(1,0) * e(3,1) - e(3,0) * e(1,1);
		const float s23 = e(1,0) * e(2,1) - e(2,0) * e(1,1);

		const float f0[4] = { s00, s00, s02, s03 };
		const float f1[4] = { s04, s04, s06, s07 };
		const float f2[4] = { s08, s08, s10, s11 };
		const float f3[4] = { s12, s12, s14, s15 };
		const float f4[4] = { s16, s16, s18, s19 };
		const float f5[4] = { s20, s20, s22, s23 };
		const float v0[4] = { e(1,0), e(0,0), e(0,0), e(0,0) };
		const float v1[4] = { e(1,1), e(0,1), e(0,1), e(0,1) };
		const float v2[4] = { e(1,2), e(0,2), e(0,2), e(0,2) };
		const float v3[4] = { e(1,3), e(0,3), e(0,3), e(0,3) };
		const float signA[4] = { +1.0f, -1.0f, +1.0f, -1.0f };
		const float signB[4] = { -1.0f, +1.0f, -1.0f, +1.0f };

		Mat4 inv;
		for (int i = 0; i < 4; ++i)
		{
			inv.at(0, i) = (v1[i] * f0[i] - v2[i] * f1[i] + v3[i] * f2[i]) * signA[i];
			inv.at(1, i) = (v0[i] * f0[i] - v2[i] * f3[i] + v3[i] * f4[i]) * signB[i];
			inv.at(2, i) = (v0[i] * f1[i] - v1[i] * f3[i] + v3[i] * f5[i]) * signA[i];
			inv.at(3, i) = (v0[i] * f2[i] - v1[i] * f4[i] + v2[i] * f5[i]) * signB[i];
		}
		const float row0[4] = { inv.at(0, 0), inv.at(1, 0), inv.at(2, 0), inv.at(3, 0) };
		float d[4];
		for (int i = 0; i < 4; ++i) d[i] = e(0, i) * row0[i];
		const float det = (d[0] + d[1]) + (d[2] + d[3]);
		const float rdet = 1.0f / det;
		for (float& v : inv.m) v = v * rdet;
		return inv;
	}

	bool AABB::Degenerate() const
	{
		for (int i = 0; i < 3; ++i)
		{
			if (std::isinf(Min[i]) || std::isinf(Max[i]) || std::isnan(Min[i]) || std::isnan(Max[i])) return true;
			if (Max[i] <= Min[i]) return true;
		}
		return false;
	}

	// Smallest cube sharing the box's centre (aabb.cpp:122-139).
	AABB AABB::BoundingCube() const
	{
		if (Degenerate()) return { Vec3(0.0f), Vec3(0.0f) };
		const Vec3 e = Max - Min;
		const float longest = std::fmax(std::fmax(e.x, e.y), e.z);
		const Vec3 pad = (Vec3(longest) - e) * Vec3(0.5f);
		return { Min - pad, Max + pad };
	}

	float AABB::Volume() const
	{
		if (Degenerate()) return 0.0f;
		const Vec3 e = Max - Min;
		return e.x * e.y * e.z;
	}

	// translate(I, T) * scale(S) * rotation(R)  (transform.cpp:49-55).
	Mat4 Transform::ToMatrix() const
	{
		const Mat4 r = MatFromQuat(Rotation);
		const Mat4 id = Mat4::Identity();
		Mat4 t = id;
		for (int i = 0; i < 4; ++i)
		{
			float a = id.at(0, i) * Translation.x;
			a = a + id.at(1, i) * Translation.y;
			a = a + id.at(2, i) * Translation.z;
			a = a + id.at(3, i);
			t.at(3, i) = a;
		}
		Mat4 s = Mat4::Identity();
		s.at(0, 0) = Scalation;
		s.at(1, 1) = Scalation;
		s.at(2, 2) = Scalation;
		const Mat4 ts = MatMul(t, s);
		return MatMul(ts, r);
	}

	// World bounds of a transformed local box: the box's 8 corners mapped through the
	// transform when it rotates, else a scale and offset (sdf_evaluator.cpp:367-406).
	AABB Transform::ApplyBounds(const AABB& in) const
	{
		if (Rotation.IsIdentity())
		{
			return { (in.Min * Scalation) + Translation, (in.Max * Scalation) + Translation };
		}
		const Vec3 A = in.Min, B = in.Max;
		const Vec3 corners[7] = {
			B, Vec3(B.x, A.y, A.z), Vec3(A.x, B.y, A.z), Vec3(A.x, A.y, B.z),
			Vec3(A.x, B.y, B.z), Vec3(B.x, A.y, B.z), Vec3(B.x, B.y, A.z) };
		AABB out;
		out.Min = Apply(A);
		out.Max = out.Min;
		for (const Vec3& c : corners)
		{
			const Vec3 q = Apply(c);
			out.Min = TernaryMin(out.Min, q);
			out.Max = TernaryMax(out.Max, q);
		}
		return out;
	}
}
