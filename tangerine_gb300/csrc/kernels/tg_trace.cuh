// Sphere-tracing pieces shared by the renderers (tg_trace.cu) and the network-stepped
// renderer (tg_field.cu): SDFNode::RayMarch's loop and SDFNode::Gradient / GetMaterial on
// the whole tree.
#pragma once

#include <cmath>

#include "tg_device.cuh"
#include "tg_kernels.hpp"

namespace tg
{
	// The whole tree's (or a cell's) surface program at one point; `spill` is this thread's
	// column of the operand stack (stride = threads in the block).
	__device__ __forceinline__ float TraceSurfaceAt(const DeviceProgram& prog, int pc, Vec3 p, bool material, int* m, float* spill,
		int stride)
	{
		const float px[1] = { p.x }, py[1] = { p.y }, pz[1] = { p.z };
		float e[1];
		RunSurfaceBatch<1>(prog.Code, pc, px, py, pz, e, material ? 0 : -1, m, spill, stride);
		return e[0];
	}

	// SDFNode::Gradient (sdf_evaluator.cpp:298-333) and, with colours, GetMaterial.
	__device__ __forceinline__ Vec3 TraceShade(const DeviceProgram& prog, int pc, Vec3 p, bool material, int* m, float* spill, int stride)
	{
		const float h = 0.0001f;
		const Vec3 xyy(h, -h, -h), yyx(-h, -h, h), yxy(-h, h, -h), xxx(h, h, h);
		const float e0 = TraceSurfaceAt(prog, pc, p + xyy, false, nullptr, spill, stride);
		const float e1 = TraceSurfaceAt(prog, pc, p + yyx, false, nullptr, spill, stride);
		const float e2 = TraceSurfaceAt(prog, pc, p + yxy, false, nullptr, spill, stride);
		const float e3 = TraceSurfaceAt(prog, pc, p + xxx, false, nullptr, spill, stride);
		Vec3 g = xyy * e0;
		g = g + yyx * e1;
		g = g + yxy * e2;
		g = g + xxx * e3;
		const float ls = (g.x * g.x + g.y * g.y) + g.z * g.z;
		if (material) TraceSurfaceAt(prog, pc, p, true, m, spill, stride);
		if (ls == 0.0f)
		{
			const float d = TraceSurfaceAt(prog, pc, p, false, nullptr, spill, stride);
			return Normalize(Vec3(e0 - d, e2 - d, e1 - d));
		}
		return g / sqrtf(ls);
	}

	struct March
	{
		bool Hit;
		float Travel;
		Vec3 Position;
	};

	// SDFNode::RayMarch on the whole tree (sdf_evaluator.cpp:336-353), starting at travel t0
	// (0: the reference's loop exactly) along the normalised direction.
	__device__ __forceinline__ March TraceExactFrom(const DeviceProgram& prog, Vec3 start, Vec3 dir, float t0, int iterations,
		float epsilon, float* spill, int stride)
	{
		Vec3 pos = t0 == 0.0f ? start : dir * t0 + start;
		float travel = t0;
		for (int i = 0; i < iterations; ++i)
		{
			const float d = TraceSurfaceAt(prog, prog.FullSurfaceCode, pos, false, nullptr, spill, stride);
			if (d <= epsilon) return { true, travel, pos };
			travel = travel + d;
			pos = dir * travel + start;
		}
		return { false, INFINITY, pos };
	}

	// Distance from p to the root cube (0 inside), the cube's centre and half-width.
	__device__ __forceinline__ float RootCubeDistance(const DeviceProgram& prog, Vec3 p)
	{
		const float half = fabsf(__ldg(&prog.Nodes[0].ClipRadius)) * 0.57735f;
		const float ox = fmaxf(fabsf(p.x - __ldg(&prog.Nodes[0].Pivot[0])) - half, 0.0f);
		const float oy = fmaxf(fabsf(p.y - __ldg(&prog.Nodes[0].Pivot[1])) - half, 0.0f);
		const float oz = fmaxf(fabsf(p.z - __ldg(&prog.Nodes[0].Pivot[2])) - half, 0.0f);
		return sqrtf(ox * ox + oy * oy + oz * oz);
	}

	// Travel at which the ray leaves the root sphere (negative: never inside it).
	__device__ __forceinline__ float RootSphereExit(const DeviceProgram& prog, Vec3 start, Vec3 dir)
	{
		const float rootClip = fabsf(__ldg(&prog.Nodes[0].ClipRadius));
		const Vec3 root(__ldg(&prog.Nodes[0].Pivot[0]), __ldg(&prog.Nodes[0].Pivot[1]), __ldg(&prog.Nodes[0].Pivot[2]));
		const Vec3 oc = start - root;
		const float b = Dot(oc, dir);
		const float c = Dot(oc, oc) - rootClip * rootClip;
		const float disc = b * b - c;
		if (disc < 0.0f) return -1.0f;
		return -b + sqrtf(disc);
	}
}
