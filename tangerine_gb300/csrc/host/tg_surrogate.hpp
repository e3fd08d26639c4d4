// Learned distance bound of one tree: a hash-grid network (kernels in tg_field.cu) trained
// on distances the exact whole-tree program produces, then used to skip export bricks.
// The exact program has the last word: every kept brick is evaluated exactly, and the
// network's error on held-out samples sets the safety margin of every skip.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "tg_engine.hpp"

namespace tg
{
	struct FieldOptions
	{
		int Log2Table = 18;             // entries per level = 2^Log2Table
		int BaseRes = 16;               // cells per axis of the coarsest level
		int MaxRes = 1024;              // of the finest level
		float Lo[3] = { -2.0f, -2.0f, -2.0f };
		float Hi[3] = { 2.0f, 2.0f, 2.0f };
		float Clamp = 0.5f;             // targets are clamp(d, -Clamp, Clamp)
		int64_t Samples = int64_t(1) << 22;     // training set: half uniform, half |d| < Band
		float Band = 0.05f;
		int64_t Batch = int64_t(1) << 18;
		int Steps = 1000;
		float Rate = 1e-2f;             // Adam step; decays to 1/10 over the last half
		float Beta1 = 0.9f, Beta2 = 0.99f, Epsilon = 1e-15f;
		int64_t Validation = int64_t(1) << 20;  // held-out samples, same mix
		float Safety = 2.0f;            // margin = Safety * max held-out error
		uint64_t Seed = 1;
	};

	struct FieldInfo
	{
		float MaxError = 0, P99Error = 0, MeanError = 0, Margin = 0, FinalLoss = 0;
		float MarginOverride = -1.0f;   // >= 0: fixed margin for every brick size
		double DataSeconds = 0, TrainSeconds = 0;
		int64_t Samples = 0;
		int Steps = 0;
	};

	class FieldNet
	{
	public:
		FieldOptions Opt;
		FieldGrid Grid{};
		FieldInfo Info;
		int64_t TableFloats = 0;

		explicit FieldNet(const FieldOptions& opt);
		~FieldNet();

		// Allocates the parameters and sets their seeded initial values.
		cudaError_t Init(cudaStream_t s);
		cudaError_t SetParams(const float* host_table, const float* host_mlp, cudaStream_t s);
		cudaError_t GetParams(float* host_table, float* host_mlp, cudaStream_t s);
		// Checkpoint: the grid options, the step count, the info and held-out error record,
		// the parameters and both Adam moments (byte layout in tg_surrogate.cpp).  Load
		// requires the same grid options; training then resumes where it stopped.
		cudaError_t Save(std::vector<uint8_t>& out, cudaStream_t s);
		cudaError_t Load(const uint8_t* data, size_t size, std::string& error, cudaStream_t s);
		// Gradients of the mean squared error over n device samples (x, y, z, d), to host.
		cudaError_t Gradients(const float4* samples, int64_t n, float* host_table_grad, float* host_mlp_grad, float* host_loss,
			cudaStream_t s);
		// `steps` Adam steps over consecutive batches of n device samples.
		cudaError_t Train(const float4* samples, int64_t n, int steps, cudaStream_t s);
		// Network output at n device points (stride floats apart) into device `out`.
		cudaError_t Eval(const float* points, int64_t n, int stride, float* out, cudaStream_t s);
		// Training set from the exact program, training, held-out error and margin.
		cudaError_t Fit(const Program& p, cudaStream_t s);
		// Samples (x, y, z, whole-tree distance): half uniform over the domain, half with
		// |d| < Band, interleaved; deterministic for a seed.
		cudaError_t MakeSamples(const Program& p, uint64_t seed, int64_t n, float4* out, cudaStream_t s);

		const float2* TablePtr() const { return Table.As<float2>(); }
		const uint8_t* ImagePtr() const { return Image.As<uint8_t>(); }
		int* StatusPtr() const { return Status.As<int>(); }
		cudaError_t CheckStatus(cudaStream_t s);
		// Margin of the brick test |net(c)| > r + m for ball radius r.  The test is wrong
		// only for a centre with |d| <= r and |net| > r + m, so the held-out samples with
		// |clamp(d)| <= r decide: m = Safety x max(max over them of |net| - r, P99Error).
		float MarginFor(float radius) const;
		int DeviceId = 0;

	private:
		cudaError_t Step(const float4* samples, int64_t n, float rate, cudaStream_t s);
		DeviceBuffer Table, TableGrad, TableM, TableV, Mlp, MlpGrad, MlpM, MlpV, Image, Status, Loss;
		int Steps = 0;
		std::vector<float> HeldAbsTarget;       // held-out |clamp(d)|, ascending
		std::vector<float> HeldPrefixMax;       // max |net| over the first i + 1 of them
	};
}

struct tg_surrogate : public tg::FieldNet
{
	using tg::FieldNet::FieldNet;
};
