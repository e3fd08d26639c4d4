#include "tg_pool.hpp"

#include <algorithm>
#include <chrono>

#include <sched.h>

namespace tg
{
	WorkerPool& WorkerPool::Get()
	{
		static WorkerPool pool;
		return pool;
	}

	namespace
	{
		// The CPUs this process may run on (a container's CPU set can be smaller than the
		// machine, which is all hardware_concurrency counts): polling workers beyond them
		// would take the cores from the ones that work.
		unsigned UsableCpus()
		{
			cpu_set_t set;
			CPU_ZERO(&set);
			if (sched_getaffinity(0, sizeof set, &set) == 0)
			{
				const int n = CPU_COUNT(&set);
				if (n > 0) return (unsigned)n;
			}
			return std::thread::hardware_concurrency();
		}
	}

	WorkerPool::WorkerPool()
	{
		const unsigned hw = UsableCpus();
		const int n = (int)std::min(hw > 1 ? hw - 1 : 1u, 31u);
		for (int i = 0; i < n; ++i) Threads.emplace_back([this]() { Run(); });
	}

	WorkerPool::~WorkerPool()
	{
		{
			std::lock_guard<std::mutex> lock(M);
			Stop.store(true);
		}
		Wake.notify_all();
		for (auto& t : Threads) t.join();
		{
			std::lock_guard<std::mutex> lock(LaterMutex);
			LaterStop = true;
		}
		LaterWake.notify_all();
		if (Background.joinable()) Background.join();
	}

	void WorkerPool::Later(std::function<void()> task)
	{
		std::lock_guard<std::mutex> lock(LaterMutex);
		LaterTasks.push_back(std::move(task));
		if (!Background.joinable())
		{
			Background = std::thread([this]()
			{
				std::vector<std::function<void()>> run;
				for (;;)
				{
					{
						std::unique_lock<std::mutex> lk(LaterMutex);
						LaterWake.wait(lk, [&]() { return LaterStop || !LaterTasks.empty(); });
						if (LaterTasks.empty()) return;   // stopping with nothing left
						run.swap(LaterTasks);
					}
					for (auto& t : run) t();
					run.clear();
				}
			});
		}
		LaterWake.notify_one();
	}

	void WorkerPool::Drain(Job& job)
	{
		int done = 0;
		for (;;)
		{
			const int i = job.Next.fetch_add(1, std::memory_order_relaxed);
			if (i >= job.Count) break;
			(*job.Body)(i);
			++done;
		}
		if (done) job.Finished.fetch_add(done, std::memory_order_acq_rel);
	}

	namespace
	{
		// How long a worker polls for the next loop before it sleeps.
		constexpr auto kPollFor = std::chrono::microseconds(300);
	}

	void WorkerPool::Run()
	{
		uint64_t seen = 0;
		for (;;)
		{
			if (Generation.load(std::memory_order_acquire) == seen)
			{
				const auto until = std::chrono::steady_clock::now() + kPollFor;
				for (int n = 1; Generation.load(std::memory_order_acquire) == seen && !Stop.load(std::memory_order_relaxed); ++n)
				{
					if ((n & 255) == 0 && std::chrono::steady_clock::now() > until) break;
				}
			}
			std::shared_ptr<Job> job;
			{
				std::unique_lock<std::mutex> lock(M);
				Wake.wait(lock, [&]() { return Stop.load() || Generation.load() != seen; });
				if (Stop.load()) return;
				seen = Generation.load();
				job = Current;
			}
			if (job) Drain(*job);
		}
	}

	void WorkerPool::ParallelFor(int count, const std::function<void(int)>& body)
	{
		if (count <= 0) return;
		std::unique_lock<std::mutex> busy(Busy, std::try_to_lock);
		if (!busy.owns_lock() || count == 1 || Threads.empty())
		{
			for (int i = 0; i < count; ++i) body(i);
			return;
		}
		auto job = std::make_shared<Job>();
		job->Body = &body;
		job->Count = count;
		{
			std::lock_guard<std::mutex> lock(M);
			Current = job;
			Generation.fetch_add(1, std::memory_order_release);
		}
		Wake.notify_all();
		Drain(*job);
		// The indices other threads claimed: once they are done nothing calls `body` again
		// (a late worker finds Next past Count).
		while (job->Finished.load(std::memory_order_acquire) != count) std::this_thread::yield();
		std::lock_guard<std::mutex> lock(M);
		if (Current == job) Current.reset();
	}
}
