// A process-wide pool of worker threads for the host side of compilation (the export
// octree's clips).  Threads are created once; ParallelFor hands out loop indices through
// one atomic counter and the calling thread works too.  One loop runs on the pool at a
// time: a caller that finds it busy runs its loop alone.
#pragma once

#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace tg
{
	class WorkerPool
	{
	public:
		static WorkerPool& Get();
		void ParallelFor(int count, const std::function<void(int)>& body);
		int Workers() const { return (int)Threads.size(); }
		~WorkerPool();

	private:
		WorkerPool();
		void Run();
		void Drain();

		std::vector<std::thread> Threads;
		std::mutex Busy;                    // held by the thread whose loop is running
		std::mutex M;
		std::condition_variable Wake, Done;
		const std::function<void(int)>* Body = nullptr;
		std::atomic<int> Next{ 0 };
		int Count = 0;
		int Active = 0;
		uint64_t Generation = 0;
		bool Stop = false;
	};
}
