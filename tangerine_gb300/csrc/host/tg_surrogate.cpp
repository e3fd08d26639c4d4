#include "tg_surrogate.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#define TG_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) return _e; } while (0)

namespace tg
{
	namespace
	{
		// splitmix64 (Steele, Lea and Flood 2014): seeds and initial parameters.
		struct SplitMix
		{
			uint64_t State;
			uint64_t Next()
			{
				uint64_t z = (State += 0x9E3779B97F4A7C15ull);
				z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
				z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
				return z ^ (z >> 31);
			}
			float Uniform(float lo, float hi)   // [lo, hi), 24-bit resolution
			{
				const float u = static_cast<float>(Next() >> 40) * (1.0f / 16777216.0f);
				return lo + (hi - lo) * u;
			}
		};

		uint64_t SubSeed(uint64_t seed, uint64_t tag)
		{
			SplitMix m{ seed ^ (tag * 0xD1B54A32D192ED03ull) };
			return m.Next();
		}

		double Seconds(std::chrono::steady_clock::time_point a)
		{
			return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
		}
	}

	FieldNet::FieldNet(const FieldOptions& opt) : Opt(opt) {}

	FieldNet::~FieldNet()
	{
		int prev = 0;
		const bool switched = cudaGetDevice(&prev) == cudaSuccess && prev != DeviceId && cudaSetDevice(DeviceId) == cudaSuccess;
		for (DeviceBuffer* b : { &Table, &TableGrad, &TableM, &TableV, &Mlp, &MlpGrad, &MlpM, &MlpV, &Image, &Status, &Loss }) b->Release();
		if (switched) cudaSetDevice(prev);
	}

	cudaError_t FieldNet::Init(cudaStream_t s)
	{
		TG_TRY(cudaGetDevice(&DeviceId));
		const int L = kFieldLevels;
		for (int a = 0; a < 3; ++a)
		{
			Grid.Lo[a] = Opt.Lo[a];
			Grid.Scale[a] = 1.0f / (Opt.Hi[a] - Opt.Lo[a]);
		}
		Grid.TableSize = 1u << Opt.Log2Table;
		Grid.Clamp = Opt.Clamp;
		Grid.DenseLevels = 0;
		const double growth = std::exp((std::log((double)Opt.MaxRes) - std::log((double)Opt.BaseRes)) / (L - 1));
		for (int l = 0; l < L; ++l)
		{
			const int r = (int)std::floor((double)Opt.BaseRes * std::pow(growth, l) + 1e-6);
			Grid.Res[l] = std::max(r, 1);
			const double corners = std::pow((double)Grid.Res[l] + 1.0, 3.0);
			if (corners <= (double)Grid.TableSize) Grid.DenseLevels |= 1u << l;
		}
		TableFloats = (int64_t)L * Grid.TableSize * 2;
		const size_t tb = (size_t)TableFloats * sizeof(float);
		const size_t mb = (size_t)kFieldParams * sizeof(float);
		for (DeviceBuffer* b : { &Table, &TableGrad, &TableM, &TableV }) TG_TRY(b->Reserve(tb));
		for (DeviceBuffer* b : { &Mlp, &MlpGrad, &MlpM, &MlpV }) TG_TRY(b->Reserve(mb));
		TG_TRY(Image.Reserve(kImageBytes));
		TG_TRY(Status.Reserve(sizeof(int)));
		TG_TRY(Loss.Reserve(sizeof(float)));
		for (DeviceBuffer* b : { &TableGrad, &TableM, &TableV }) TG_TRY(cudaMemsetAsync(b->Ptr, 0, tb, s));
		for (DeviceBuffer* b : { &MlpGrad, &MlpM, &MlpV }) TG_TRY(cudaMemsetAsync(b->Ptr, 0, mb, s));
		TG_TRY(cudaMemsetAsync(Status.Ptr, 0, sizeof(int), s));
		TG_TRY(cudaMemsetAsync(Loss.Ptr, 0, sizeof(float), s));

		// Table U(-1e-4, 1e-4); weights Glorot-uniform; biases zero.
		SplitMix rng{ SubSeed(Opt.Seed, 1) };
		std::vector<float> table((size_t)TableFloats);
		for (float& x : table) x = rng.Uniform(-1e-4f, 1e-4f);
		std::vector<float> mlp(kFieldParams, 0.0f);
		auto glorot = [&](int off, int out, int in) {
			const float a = std::sqrt(6.0f / (float)(in + out));
			for (int i = 0; i < out * in; ++i) mlp[off + i] = rng.Uniform(-a, a);
		};
		glorot(kFieldW1, 64, 32);
		glorot(kFieldW2, 64, 64);
		glorot(kFieldW3, 64, 64);
		glorot(kFieldW4, 1, 64);
		Steps = 0;
		return SetParams(table.data(), mlp.data(), s);
	}

	cudaError_t FieldNet::SetParams(const float* host_table, const float* host_mlp, cudaStream_t s)
	{
		if (host_table) TG_TRY(cudaMemcpyAsync(Table.Ptr, host_table, (size_t)TableFloats * sizeof(float), cudaMemcpyHostToDevice, s));
		if (host_mlp) TG_TRY(cudaMemcpyAsync(Mlp.Ptr, host_mlp, (size_t)kFieldParams * sizeof(float), cudaMemcpyHostToDevice, s));
		TG_TRY(LaunchFieldPack(Mlp.As<float>(), Image.As<uint8_t>(), s));
		return cudaStreamSynchronize(s);
	}

	cudaError_t FieldNet::GetParams(float* host_table, float* host_mlp, cudaStream_t s)
	{
		if (host_table) TG_TRY(cudaMemcpyAsync(host_table, Table.Ptr, (size_t)TableFloats * sizeof(float), cudaMemcpyDeviceToHost, s));
		if (host_mlp) TG_TRY(cudaMemcpyAsync(host_mlp, Mlp.Ptr, (size_t)kFieldParams * sizeof(float), cudaMemcpyDeviceToHost, s));
		return cudaStreamSynchronize(s);
	}

	// Checkpoint bytes, little-endian, in this order: the magic "TGFIELD1"; int32 Log2Table,
	// BaseRes, MaxRes; float Lo[3], Hi[3], Clamp; int64 table floats; int32 network floats;
	// int32 steps taken; the info (float MaxError, P99Error, MeanError, Margin, FinalLoss,
	// MarginOverride; double DataSeconds, TrainSeconds; int64 Samples; int32 Steps); int64
	// held-out count; then float arrays: table, its first and second moments, network, its
	// two moments, the held-out |clamp(d)| and prefix maxima.
	namespace
	{
		constexpr char kCheckpointMagic[8] = { 'T', 'G', 'F', 'I', 'E', 'L', 'D', '1' };

		struct Writer
		{
			std::vector<uint8_t>& Out;
			template<typename T> void Put(const T& v)
			{
				const uint8_t* b = reinterpret_cast<const uint8_t*>(&v);
				Out.insert(Out.end(), b, b + sizeof(T));
			}
		};

		struct Reader
		{
			const uint8_t* At;
			const uint8_t* End;
			template<typename T> bool Get(T& v)
			{
				if ((size_t)(End - At) < sizeof(T)) return false;
				std::memcpy(&v, At, sizeof(T));
				At += sizeof(T);
				return true;
			}
		};
	}

	cudaError_t FieldNet::Save(std::vector<uint8_t>& out, cudaStream_t s)
	{
		out.clear();
		Writer w{ out };
		for (char c : kCheckpointMagic) w.Put(c);
		w.Put((int32_t)Opt.Log2Table); w.Put((int32_t)Opt.BaseRes); w.Put((int32_t)Opt.MaxRes);
		for (int i = 0; i < 3; ++i) w.Put(Opt.Lo[i]);
		for (int i = 0; i < 3; ++i) w.Put(Opt.Hi[i]);
		w.Put(Opt.Clamp);
		w.Put((int64_t)TableFloats); w.Put((int32_t)kFieldParams);
		w.Put((int32_t)Steps);
		w.Put(Info.MaxError); w.Put(Info.P99Error); w.Put(Info.MeanError); w.Put(Info.Margin); w.Put(Info.FinalLoss);
		w.Put(Info.MarginOverride); w.Put(Info.DataSeconds); w.Put(Info.TrainSeconds); w.Put((int64_t)Info.Samples);
		w.Put((int32_t)Info.Steps);
		const int64_t held = (int64_t)HeldAbsTarget.size();
		w.Put(held);
		const size_t head = out.size();
		const size_t tb = (size_t)TableFloats * 4, mb = (size_t)kFieldParams * 4, hb = (size_t)held * 4;
		out.resize(head + 3 * tb + 3 * mb + 2 * hb);
		uint8_t* p = out.data() + head;
		const DeviceBuffer* tables[3] = { &Table, &TableM, &TableV };
		for (const DeviceBuffer* b : tables) { TG_TRY(cudaMemcpyAsync(p, b->Ptr, tb, cudaMemcpyDeviceToHost, s)); p += tb; }
		const DeviceBuffer* nets[3] = { &Mlp, &MlpM, &MlpV };
		for (const DeviceBuffer* b : nets) { TG_TRY(cudaMemcpyAsync(p, b->Ptr, mb, cudaMemcpyDeviceToHost, s)); p += mb; }
		if (held)
		{
			std::memcpy(p, HeldAbsTarget.data(), hb);
			std::memcpy(p + hb, HeldPrefixMax.data(), hb);
		}
		return cudaStreamSynchronize(s);
	}

	cudaError_t FieldNet::Load(const uint8_t* data, size_t size, std::string& error, cudaStream_t s)
	{
		Reader r{ data, data + size };
		char magic[8];
		for (char& c : magic)
			if (!r.Get(c)) { error = "checkpoint too short"; return cudaErrorInvalidValue; }
		if (std::memcmp(magic, kCheckpointMagic, 8) != 0) { error = "not a surrogate checkpoint"; return cudaErrorInvalidValue; }
		int32_t log2Table = 0, baseRes = 0, maxRes = 0, mlpFloats = 0, steps = 0, infoSteps = 0;
		float lo[3], hi[3], clamp = 0.0f;
		int64_t tableFloats = 0, samples = 0, held = 0;
		FieldInfo info;
		bool ok = r.Get(log2Table) && r.Get(baseRes) && r.Get(maxRes);
		for (int i = 0; i < 3; ++i) ok = ok && r.Get(lo[i]);
		for (int i = 0; i < 3; ++i) ok = ok && r.Get(hi[i]);
		ok = ok && r.Get(clamp) && r.Get(tableFloats) && r.Get(mlpFloats) && r.Get(steps);
		ok = ok && r.Get(info.MaxError) && r.Get(info.P99Error) && r.Get(info.MeanError) && r.Get(info.Margin) && r.Get(info.FinalLoss)
			&& r.Get(info.MarginOverride) && r.Get(info.DataSeconds) && r.Get(info.TrainSeconds) && r.Get(samples) && r.Get(infoSteps)
			&& r.Get(held);
		if (!ok) { error = "checkpoint too short"; return cudaErrorInvalidValue; }
		bool same = log2Table == Opt.Log2Table && baseRes == Opt.BaseRes && maxRes == Opt.MaxRes && clamp == Opt.Clamp;
		for (int i = 0; i < 3; ++i) same = same && lo[i] == Opt.Lo[i] && hi[i] == Opt.Hi[i];
		if (!same || tableFloats != TableFloats || mlpFloats != kFieldParams)
		{
			error = "checkpoint of a surrogate with other grid options";
			return cudaErrorInvalidValue;
		}
		const size_t tb = (size_t)TableFloats * 4, mb = (size_t)kFieldParams * 4;
		if (held < 0 || steps < 0 || (size_t)(r.End - r.At) != 3 * tb + 3 * mb + 2 * (size_t)held * 4)
		{
			error = "checkpoint size does not match its header";
			return cudaErrorInvalidValue;
		}
		const uint8_t* p = r.At;
		DeviceBuffer* tables[3] = { &Table, &TableM, &TableV };
		for (DeviceBuffer* b : tables) { TG_TRY(cudaMemcpyAsync(b->Ptr, p, tb, cudaMemcpyHostToDevice, s)); p += tb; }
		DeviceBuffer* nets[3] = { &Mlp, &MlpM, &MlpV };
		for (DeviceBuffer* b : nets) { TG_TRY(cudaMemcpyAsync(b->Ptr, p, mb, cudaMemcpyHostToDevice, s)); p += mb; }
		TG_TRY(cudaMemsetAsync(TableGrad.Ptr, 0, tb, s));
		TG_TRY(cudaMemsetAsync(MlpGrad.Ptr, 0, mb, s));
		TG_TRY(LaunchFieldPack(Mlp.As<float>(), Image.As<uint8_t>(), s));
		HeldAbsTarget.resize((size_t)held);
		HeldPrefixMax.resize((size_t)held);
		if (held)
		{
			std::memcpy(HeldAbsTarget.data(), p, (size_t)held * 4);
			std::memcpy(HeldPrefixMax.data(), p + (size_t)held * 4, (size_t)held * 4);
		}
		Steps = steps;
		info.Samples = samples;
		info.Steps = infoSteps;
		Info = info;
		return cudaStreamSynchronize(s);
	}

	cudaError_t FieldNet::CheckStatus(cudaStream_t s)
	{
		int st = 0;
		TG_TRY(cudaMemcpyAsync(&st, Status.Ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaStreamSynchronize(s));
		if (st != 0)
		{
			cudaMemsetAsync(Status.Ptr, 0, sizeof(int), s);
			return cudaErrorLaunchTimeout;
		}
		return cudaSuccess;
	}

	cudaError_t FieldNet::Gradients(const float4* samples, int64_t n, float* host_table_grad, float* host_mlp_grad, float* host_loss,
		cudaStream_t s)
	{
		const size_t tb = (size_t)TableFloats * sizeof(float), mb = (size_t)kFieldParams * sizeof(float);
		TG_TRY(cudaMemsetAsync(TableGrad.Ptr, 0, tb, s));
		TG_TRY(cudaMemsetAsync(MlpGrad.Ptr, 0, mb, s));
		TG_TRY(cudaMemsetAsync(Loss.Ptr, 0, sizeof(float), s));
		TG_TRY(LaunchFieldTrain(Grid, Table.As<float2>(), Image.As<uint8_t>(), samples, n, TableGrad.As<float2>(), MlpGrad.As<float>(),
			Loss.As<float>(), Status.As<int>(), s));
		TG_TRY(CheckStatus(s));
		if (host_table_grad) TG_TRY(cudaMemcpyAsync(host_table_grad, TableGrad.Ptr, tb, cudaMemcpyDeviceToHost, s));
		if (host_mlp_grad) TG_TRY(cudaMemcpyAsync(host_mlp_grad, MlpGrad.Ptr, mb, cudaMemcpyDeviceToHost, s));
		if (host_loss) TG_TRY(cudaMemcpyAsync(host_loss, Loss.Ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
		TG_TRY(cudaMemsetAsync(TableGrad.Ptr, 0, tb, s));
		TG_TRY(cudaMemsetAsync(MlpGrad.Ptr, 0, mb, s));
		return cudaStreamSynchronize(s);
	}

	cudaError_t FieldNet::Step(const float4* samples, int64_t n, float rate, cudaStream_t s)
	{
		TG_TRY(LaunchFieldTrain(Grid, Table.As<float2>(), Image.As<uint8_t>(), samples, n, TableGrad.As<float2>(), MlpGrad.As<float>(),
			Loss.As<float>(), Status.As<int>(), s));
		++Steps;
		AdamStep a;
		a.Rate = rate;
		a.Beta1 = Opt.Beta1;
		a.Beta2 = Opt.Beta2;
		a.Epsilon = Opt.Epsilon;
		a.Correction1 = (float)(1.0 - std::pow((double)Opt.Beta1, Steps));
		a.Correction2 = (float)(1.0 - std::pow((double)Opt.Beta2, Steps));
		TG_TRY(LaunchAdam(Table.As<float>(), TableGrad.As<float>(), TableM.As<float>(), TableV.As<float>(), TableFloats, a, s));
		TG_TRY(LaunchAdam(Mlp.As<float>(), MlpGrad.As<float>(), MlpM.As<float>(), MlpV.As<float>(), kFieldParams, a, s));
		return LaunchFieldPack(Mlp.As<float>(), Image.As<uint8_t>(), s);
	}

	cudaError_t FieldNet::Train(const float4* samples, int64_t n, int steps, cudaStream_t s)
	{
		if (n <= 0 || steps <= 0) return cudaSuccess;
		const int64_t batch = std::min<int64_t>(Opt.Batch, n);
		float lastLoss = 0.0f;
		int64_t lastCount = 0;
		int64_t offset = 0;
		for (int i = 0; i < steps; ++i)
		{
			const double progress = (double)i / (double)steps;
			const float rate = progress < 0.5 ? Opt.Rate : (float)(Opt.Rate * std::pow(0.1, (progress - 0.5) / 0.5));
			if (offset >= n) offset = 0;
			const int64_t m = std::min<int64_t>(batch, n - offset);
			if (i == steps - 1) TG_TRY(cudaMemsetAsync(Loss.Ptr, 0, sizeof(float), s));
			TG_TRY(Step(samples + offset, m, rate, s));
			if (i == steps - 1) lastCount = m;
			offset += m;
		}
		TG_TRY(cudaMemcpyAsync(&lastLoss, Loss.Ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
		TG_TRY(CheckStatus(s));
		Info.FinalLoss = lastCount ? lastLoss / (float)lastCount : 0.0f;
		Info.Steps += steps;
		return cudaSuccess;
	}

	cudaError_t FieldNet::Eval(const float* points, int64_t n, int stride, float* out, cudaStream_t s)
	{
		TG_TRY(LaunchFieldEval(Grid, Table.As<float2>(), Image.As<uint8_t>(), points, n, stride, out, Status.As<int>(), s));
		return CheckStatus(s);
	}

	cudaError_t FieldNet::MakeSamples(const Program& p, uint64_t seed, int64_t n, float4* out, cudaStream_t s)
	{
		const int64_t half = n / 2;
		const int64_t chunk = int64_t(1) << 22;
		const int64_t words = chunk / 32;
		DeviceBuffer tmp, flags, base, scratch, total;
		cudaError_t e = cudaSuccess;
		auto finish = [&](cudaError_t err) { tmp.Release(); flags.Release(); base.Release(); scratch.Release(); total.Release(); return err; };
		if ((e = tmp.Reserve((size_t)chunk * sizeof(float4))) != cudaSuccess) return finish(e);
		if ((e = flags.Reserve((size_t)words * 4)) != cudaSuccess) return finish(e);
		if ((e = base.Reserve((size_t)words * 4)) != cudaSuccess) return finish(e);
		if ((e = scratch.Reserve(ScanScratchWords(words) * 4)) != cudaSuccess) return finish(e);
		if ((e = total.Reserve(4)) != cudaSuccess) return finish(e);
		// Uniform half: even slots.
		for (int64_t done = 0, round = 0; done < n - half; ++round)
		{
			const int64_t m = std::min<int64_t>(chunk, (n - half) - done);
			if ((e = LaunchFieldUniform(SubSeed(seed, 0x100 + round), Opt.Lo, Opt.Hi, tmp.As<float4>(), m, 1, 0, s)) != cudaSuccess) return finish(e);
			if ((e = LaunchEvalFull(p.View, tmp.As<float4>(), m, s)) != cudaSuccess) return finish(e);
			if ((e = cudaMemcpy2DAsync(out + 2 * done, 2 * sizeof(float4), tmp.Ptr, sizeof(float4), sizeof(float4), (size_t)m,
				cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return finish(e);
			done += m;
		}
		// Near-surface half: odd slots, rejection sampled in order.
		int64_t collected = 0;
		for (int round = 0; collected < half; ++round)
		{
			if (round >= 1024)
			{
				SetError("surrogate training data: too few samples near the surface (is the tree empty?)");
				return finish(cudaErrorInvalidValue);
			}
			if ((e = LaunchFieldUniform(SubSeed(seed, 0x200000 + round), Opt.Lo, Opt.Hi, tmp.As<float4>(), chunk, 1, 0, s)) != cudaSuccess) return finish(e);
			if ((e = LaunchEvalFull(p.View, tmp.As<float4>(), chunk, s)) != cudaSuccess) return finish(e);
			if ((e = LaunchBandFlags(tmp.As<float4>(), chunk, Opt.Band, flags.As<uint32_t>(), s)) != cudaSuccess) return finish(e);
			if ((e = LaunchExclusiveScan(flags.As<uint32_t>(), words, true, base.As<uint32_t>(), total.As<uint32_t>(),
				scratch.As<uint32_t>(), s)) != cudaSuccess) return finish(e);
			if ((e = LaunchBandCompact(tmp.As<float4>(), chunk, flags.As<uint32_t>(), base.As<uint32_t>(), out, collected, half, 2, 1, s))
				!= cudaSuccess) return finish(e);
			uint32_t got = 0;
			if ((e = cudaMemcpyAsync(&got, total.Ptr, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return finish(e);
			if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return finish(e);
			collected += got;
		}
		return finish(cudaStreamSynchronize(s));
	}

	cudaError_t FieldNet::Fit(const Program& p, cudaStream_t s)
	{
		const int64_t n = Opt.Samples & ~int64_t(1);
		const int64_t nv = Opt.Validation & ~int64_t(1);
		if (n < 2 || nv < 2) return cudaErrorInvalidValue;
		DeviceBuffer data, val, pred;
		auto done = [&](cudaError_t err) { data.Release(); val.Release(); pred.Release(); return err; };
		cudaError_t e;
		auto t0 = std::chrono::steady_clock::now();
		if ((e = data.Reserve((size_t)n * sizeof(float4))) != cudaSuccess) return done(e);
		if ((e = MakeSamples(p, SubSeed(Opt.Seed, 2), n, data.As<float4>(), s)) != cudaSuccess) return done(e);
		Info.DataSeconds = Seconds(t0);
		Info.Samples = n;
		auto t1 = std::chrono::steady_clock::now();
		if ((e = Train(data.As<float4>(), n, Opt.Steps, s)) != cudaSuccess) return done(e);
		if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return done(e);
		Info.TrainSeconds = Seconds(t1);
		data.Release();

		// Held-out error against clamp(d) and the margin every skip is widened by.
		if ((e = val.Reserve((size_t)nv * sizeof(float4))) != cudaSuccess) return done(e);
		if ((e = pred.Reserve((size_t)nv * sizeof(float))) != cudaSuccess) return done(e);
		if ((e = MakeSamples(p, SubSeed(Opt.Seed, 3), nv, val.As<float4>(), s)) != cudaSuccess) return done(e);
		if ((e = Eval(val.As<float>(), nv, 4, pred.As<float>(), s)) != cudaSuccess) return done(e);
		std::vector<float4> hv((size_t)nv);
		std::vector<float> hp((size_t)nv);
		if ((e = cudaMemcpyAsync(hv.data(), val.Ptr, (size_t)nv * sizeof(float4), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return done(e);
		if ((e = cudaMemcpyAsync(hp.data(), pred.Ptr, (size_t)nv * sizeof(float), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return done(e);
		if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return done(e);
		std::vector<float> err((size_t)nv);
		double sum = 0.0;
		for (int64_t i = 0; i < nv; ++i)
		{
			const float t = std::min(std::max(hv[i].w, -Opt.Clamp), Opt.Clamp);
			err[i] = std::fabs(hp[i] - t);
			sum += err[i];
		}
		Info.MeanError = (float)(sum / (double)nv);
		Info.MaxError = *std::max_element(err.begin(), err.end());
		const size_t k = (size_t)((double)(nv - 1) * 0.99);
		std::nth_element(err.begin(), err.begin() + k, err.end());
		Info.P99Error = err[k];
		Info.Margin = Opt.Safety * Info.MaxError;
		{
			std::vector<std::pair<float, float>> ts((size_t)nv);
			for (int64_t i = 0; i < nv; ++i)
				ts[i] = { std::fabs(std::min(std::max(hv[i].w, -Opt.Clamp), Opt.Clamp)), std::fabs(hp[i]) };
			std::sort(ts.begin(), ts.end());
			HeldAbsTarget.resize((size_t)nv);
			HeldPrefixMax.resize((size_t)nv);
			float m = 0.0f;
			for (int64_t i = 0; i < nv; ++i)
			{
				HeldAbsTarget[i] = ts[i].first;
				m = std::max(m, ts[i].second);
				HeldPrefixMax[i] = m;
			}
		}
		return done(cudaSuccess);
	}

	float FieldNet::MarginFor(float radius) const
	{
		if (Info.MarginOverride >= 0.0f) return Info.MarginOverride;
		if (HeldAbsTarget.empty()) return Opt.Safety * Opt.Clamp;          // never fitted: rule nothing out
		const size_t k = (size_t)(std::upper_bound(HeldAbsTarget.begin(), HeldAbsTarget.end(), radius) - HeldAbsTarget.begin());
		const float worst = k ? std::max(HeldPrefixMax[k - 1] - radius, 0.0f) : 0.0f;
		return Opt.Safety * std::max(worst, Info.P99Error);
	}
}
