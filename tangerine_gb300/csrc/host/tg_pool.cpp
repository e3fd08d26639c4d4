#include "tg_pool.hpp"

#include <algorithm>

namespace tg
{
	WorkerPool& WorkerPool::Get()
	{
		static WorkerPool pool;
		return pool;
	}

	WorkerPool::WorkerPool()
	{
		const unsigned hw = std::thread::hardware_concurrency();
		const int n = (int)std::min(hw > 1 ? hw - 1 : 1u, 31u);
		for (int i = 0; i < n; ++i) Threads.emplace_back([this]() { Run(); });
	}

	WorkerPool::~WorkerPool()
	{
		{
			std::lock_guard<std::mutex> lock(M);
			Stop = true;
		}
		Wake.notify_all();
		for (auto& t : Threads) t.join();
	}

	void WorkerPool::Drain()
	{
		for (;;)
		{
			const int i = Next.fetch_add(1, std::memory_order_relaxed);
			if (i >= Count) return;
			(*Body)(i);
		}
	}

	void WorkerPool::Run()
	{
		uint64_t seen = 0;
		for (;;)
		{
			{
				std::unique_lock<std::mutex> lock(M);
				Wake.wait(lock, [&]() { return Stop || Generation != seen; });
				if (Stop) return;
				seen = Generation;
			}
			Drain();
			{
				std::lock_guard<std::mutex> lock(M);
				if (--Active == 0) Done.notify_all();
			}
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
		{
			std::lock_guard<std::mutex> lock(M);
			Body = &body;
			Count = count;
			Next.store(0, std::memory_order_relaxed);
			Active = (int)Threads.size();
			++Generation;
		}
		Wake.notify_all();
		Drain();
		std::unique_lock<std::mutex> lock(M);
		Done.wait(lock, [&]() { return Active == 0; });
		Body = nullptr;
	}
}
