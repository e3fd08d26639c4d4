// Sphere tracing (SDFNode::RayMarch, tangerine/sdf_evaluator.cpp:336-353) and a
// depth / normal / colour renderer built on it.
//
// Exact form: the reference's step sequence -- every step is the whole tree's distance
// (its surface program, SDFNode::Eval order) -- so hits, travel and positions are those of
// SDFNode::RayMarch bit for bit.
//
// Octree-bounded form: outside the root cube the distance to that cube is a safe step (the
// surface lies inside it).  Inside, a point lies in the cube of the octree cell Descend
// picks, and the whole tree's distance is at least min(f_cell(q), R - |q - P|): every operand
// the cell's clip dropped exceeds R - |q - P| there (1-Lipschitz), and union, diff and the
// polynomial blends cannot fall below that bound.  The cell's distance program is a few
// brushes where the full tree is hundreds.  A hit is declared when f_cell(q) <= epsilon,
// which then holds for the whole tree too.  Shading uses the cell's surface program as
// SDFOctree::Gradient / GetMaterial do.
#include <cmath>

#include "tg_device.cuh"
#include "tg_kernels.hpp"
#include "tg_trace.cuh"

namespace tg
{
	namespace
	{
		constexpr int kTraceThreads = 128;

		// SDFNode::RayMarch on the whole tree.
		__device__ __forceinline__ March MarchExact(const DeviceProgram& prog, Vec3 start, Vec3 dir_in, int iterations, float epsilon,
			float* spill)
		{
			return TraceExactFrom(prog, start, Normalize(dir_in), 0.0f, iterations, epsilon, spill, kTraceThreads);
		}

		__device__ __forceinline__ March MarchBounded(const DeviceProgram& prog, Vec3 start, Vec3 dir_in, int iterations, float epsilon,
			float* spill)
		{
			const Vec3 dir = Normalize(dir_in);
			const float rootClip = fabsf(__ldg(&prog.Nodes[0].ClipRadius));
			const Vec3 root(__ldg(&prog.Nodes[0].Pivot[0]), __ldg(&prog.Nodes[0].Pivot[1]), __ldg(&prog.Nodes[0].Pivot[2]));
			const float half = rootClip * 0.57735f;               // root cube half-width
			// Leaving the root sphere along the ray ends the march: nothing lies beyond.
			const Vec3 oc = start - root;
			const float b = Dot(oc, dir);
			const float c = Dot(oc, oc) - rootClip * rootClip;
			const float disc = b * b - c;
			if (disc < 0.0f) return { false, INFINITY, start };
			const float exitTravel = -b + sqrtf(disc);
			if (exitTravel < 0.0f) return { false, INFINITY, start };
			Vec3 pos = start;
			float travel = 0.0f;
			for (int i = 0; i < iterations; ++i)
			{
				const Vec3 off = pos - root;
				const float ox = fmaxf(fabsf(off.x) - half, 0.0f), oy = fmaxf(fabsf(off.y) - half, 0.0f), oz = fmaxf(fabsf(off.z) - half, 0.0f);
				float step = sqrtf(ox * ox + oy * oy + oz * oz);
				if (!(step > epsilon))
				{
					const int cell = DescendOctree(prog.Nodes, pos.x, pos.y, pos.z);
					const float px[1] = { pos.x }, py[1] = { pos.y }, pz[1] = { pos.z };
					float f[1];
					RunDistance<1>(prog.Code, __ldg(&prog.Nodes[cell].DistanceCode), px, py, pz, f, spill, kTraceThreads);
					if (f[0] <= epsilon) return { true, travel, pos };
					const Vec3 dp = pos - Vec3(__ldg(&prog.Nodes[cell].Pivot[0]), __ldg(&prog.Nodes[cell].Pivot[1]), __ldg(&prog.Nodes[cell].Pivot[2]));
					const float room = __ldg(&prog.Nodes[cell].ClipRadius) - Length(dp);
					step = fminf(f[0], fmaxf(room, epsilon));
				}
				travel = travel + step;
				if (travel > exitTravel) break;
				pos = dir * travel + start;
			}
			return { false, INFINITY, pos };
		}

		__global__ void __launch_bounds__(kTraceThreads) RayMarchKernel(DeviceProgram prog, const float* __restrict__ origins,
			const float* __restrict__ dirs, int64_t n, int iterations, float epsilon, uint8_t* __restrict__ hit,
			float* __restrict__ travel, float* __restrict__ position)
		{
			extern __shared__ float spill[];
			const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (r >= n) return;
			const March m = MarchExact(prog, Vec3(origins[r * 3], origins[r * 3 + 1], origins[r * 3 + 2]),
				Vec3(dirs[r * 3], dirs[r * 3 + 1], dirs[r * 3 + 2]), iterations, epsilon, spill + threadIdx.x);
			hit[r] = m.Hit ? 1 : 0;
			travel[r] = m.Travel;
			position[r * 3] = m.Position.x;
			position[r * 3 + 1] = m.Position.y;
			position[r * 3 + 2] = m.Position.z;
		}

		// The app's framed casts: mode 1 is Lua's magnet cast (lua_sdf.cpp:410-417, the
		// direction is normalize(target - origin)); mode 2 is SDFModel::RayMarch
		// (sdf_model.cpp:261-266): origin = Transform::ApplyInv (rotate by the inverse
		// rotation after removing the translation, then divide by the scale), direction
		// rotated by the inverse rotation.
		__global__ void __launch_bounds__(kTraceThreads) RayQueryKernel(DeviceProgram prog, RayFrame f, const float* __restrict__ origins,
			const float* __restrict__ dirs, int64_t n, int iterations, float epsilon, uint8_t* __restrict__ hit,
			float* __restrict__ travel, float* __restrict__ position)
		{
			extern __shared__ float spill[];
			const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (r >= n) return;
			Vec3 o(origins[r * 3], origins[r * 3 + 1], origins[r * 3 + 2]);
			Vec3 d(dirs[r * 3], dirs[r * 3 + 1], dirs[r * 3 + 2]);
			if (f.Mode == 1)
			{
				d = Normalize(d - o);
			}
			else if (f.Mode == 2)
			{
				const Quat qi = Inverse(Quat{ f.Rotation[0], f.Rotation[1], f.Rotation[2], f.Rotation[3] });
				o = Rotate(qi, o - Vec3(f.Translation[0], f.Translation[1], f.Translation[2])) / f.Scale;
				d = Rotate(qi, d);
			}
			const March m = MarchExact(prog, o, d, iterations, epsilon, spill + threadIdx.x);
			hit[r] = m.Hit ? 1 : 0;
			travel[r] = m.Travel;
			position[r * 3] = m.Position.x;
			position[r * 3 + 1] = m.Position.y;
			position[r * 3 + 2] = m.Position.z;
		}

		// SDFNode::Eval (gradient = false) or SDFNode::Gradient on the whole tree per point,
		// as Lua's eval / gradient and EvalTree compute them (lua_sdf.cpp:386-405).
		__global__ void __launch_bounds__(kTraceThreads) PointQueryKernel(DeviceProgram prog, const float* __restrict__ points, int64_t n,
			bool gradient, float* __restrict__ out)
		{
			extern __shared__ float spill[];
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (t >= n) return;
			const Vec3 p(points[t * 3], points[t * 3 + 1], points[t * 3 + 2]);
			if (gradient)
			{
				const Vec3 g = TraceShade(prog, prog.FullSurfaceCode, p, false, nullptr, spill + threadIdx.x, kTraceThreads);
				out[t * 3] = g.x;
				out[t * 3 + 1] = g.y;
				out[t * 3 + 2] = g.z;
			}
			else
			{
				out[t] = TraceSurfaceAt(prog, prog.FullSurfaceCode, p, false, nullptr, spill + threadIdx.x, kTraceThreads);
			}
		}

		// Compiled for 10 resident CTAs per SM (48 registers instead of 56): 657 -> 667 M
		// rays/s on the 1024-primitive scene; 12 (40 registers) measured 657 again.
		__global__ void __launch_bounds__(kTraceThreads, 10) RenderKernel(DeviceProgram prog, const CameraBasis* __restrict__ cams,
			int count, int width, int height, int steps, float epsilon, bool exact, float* __restrict__ depth,
			float* __restrict__ normals, uint8_t* __restrict__ colors)
		{
			extern __shared__ float spill[];
			const int64_t pixels = (int64_t)width * height;
			const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
			if (t >= pixels * count) return;
			const int c = (int)(t / pixels);
			const int64_t pix = t % pixels;
			const int x = (int)(pix % width), y = (int)(pix / width);
			const CameraBasis& cam = cams[c];
			const float u = ((2.0f * ((float)x + 0.5f) / (float)width) - 1.0f) * cam.TanHalfFov * cam.Aspect;
			const float v = (1.0f - 2.0f * ((float)y + 0.5f) / (float)height) * cam.TanHalfFov;
			const Vec3 fwd(cam.Forward[0], cam.Forward[1], cam.Forward[2]);
			const Vec3 right(cam.Right[0], cam.Right[1], cam.Right[2]);
			const Vec3 up(cam.Up[0], cam.Up[1], cam.Up[2]);
			const Vec3 dir = (fwd + right * u) + up * v;
			const Vec3 start(cam.Position[0], cam.Position[1], cam.Position[2]);
			float* my = spill + threadIdx.x;
			const March m = exact ? MarchExact(prog, start, dir, steps, epsilon, my) : MarchBounded(prog, start, dir, steps, epsilon, my);
			depth[t] = m.Travel;
			Vec3 n(0.0f, 0.0f, 0.0f);
			uchar4 col = make_uchar4(0, 0, 0, 0);
			if (m.Hit)
			{
				const int pc = exact ? prog.FullSurfaceCode
					: __ldg(&prog.Nodes[DescendOctree(prog.Nodes, m.Position.x, m.Position.y, m.Position.z)].SurfaceCode);
				int mat = -1;
				n = TraceShade(prog, pc, m.Position, colors != nullptr, &mat, my, kTraceThreads);
				col = mat >= 0 ? prog.Colors[mat] : make_uchar4(255, 255, 255, 255);
			}
			normals[t * 3] = n.x;
			normals[t * 3 + 1] = n.y;
			normals[t * 3 + 2] = n.z;
			if (colors)
			{
				colors[t * 3] = col.x;
				colors[t * 3 + 1] = col.y;
				colors[t * 3 + 2] = col.z;
			}
		}

		size_t TraceSpillBytes(const DeviceProgram& prog)
		{
			const int depth = prog.MaxStack > 1 ? prog.MaxStack - 1 : 1;
			return (size_t)depth * 2 * kTraceThreads * sizeof(float);
		}
	}

	cudaError_t LaunchRayMarch(const DeviceProgram& prog, const float* origins, const float* dirs, int64_t n, int max_iterations,
		float epsilon, uint8_t* hit, float* travel, float* position, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		const size_t smem = TraceSpillBytes(prog);
		if (smem > 48 * 1024) cudaFuncSetAttribute(RayMarchKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		RayMarchKernel<<<(unsigned)((n + kTraceThreads - 1) / kTraceThreads), kTraceThreads, smem, stream>>>(
			prog, origins, dirs, n, max_iterations, epsilon, hit, travel, position);
		return cudaGetLastError();
	}

	cudaError_t LaunchRayQuery(const DeviceProgram& prog, const RayFrame& frame, const float* origins, const float* dirs, int64_t n,
		int max_iterations, float epsilon, uint8_t* hit, float* travel, float* position, cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		const size_t smem = TraceSpillBytes(prog);
		if (smem > 48 * 1024)
		{
			cudaError_t e = cudaFuncSetAttribute(RayQueryKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		RayQueryKernel<<<(unsigned)((n + kTraceThreads - 1) / kTraceThreads), kTraceThreads, smem, stream>>>(
			prog, frame, origins, dirs, n, max_iterations, epsilon, hit, travel, position);
		return cudaGetLastError();
	}

	cudaError_t LaunchPointQuery(const DeviceProgram& prog, const float* points, int64_t n, bool gradient, float* out,
		cudaStream_t stream)
	{
		if (n <= 0) return cudaSuccess;
		const size_t smem = TraceSpillBytes(prog);
		if (smem > 48 * 1024)
		{
			cudaError_t e = cudaFuncSetAttribute(PointQueryKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
		PointQueryKernel<<<(unsigned)((n + kTraceThreads - 1) / kTraceThreads), kTraceThreads, smem, stream>>>(
			prog, points, n, gradient, out);
		return cudaGetLastError();
	}

	cudaError_t LaunchRender(const DeviceProgram& prog, const CameraBasis* cameras, int count, int width, int height,
		int max_steps, float epsilon, bool exact, float* depth, float* normals, uint8_t* colors, cudaStream_t stream)
	{
		const int64_t total = (int64_t)width * height * count;
		if (total <= 0) return cudaSuccess;
		const size_t smem = TraceSpillBytes(prog);
		if (smem > 48 * 1024) cudaFuncSetAttribute(RenderKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		RenderKernel<<<(unsigned)((total + kTraceThreads - 1) / kTraceThreads), kTraceThreads, smem, stream>>>(
			prog, cameras, count, width, height, max_steps, epsilon, exact || !prog.Lipschitz, depth, normals, colors);
		return cudaGetLastError();
	}
}
