// A process-wide pool of worker threads for the host side of compilation (the export
// octree's clips, the program emission).  Threads are created once; ParallelFor hands out
// loop indices through one atomic counter and the calling thread works too.  One loop runs
// on the pool at a time: a caller that finds it busy runs its loop alone.
//
// A compile runs several loops back to back (one per octree level, then the programs), so
// waking threads must not sit on the critical path.  The caller waits for the indices to
// be done, not for every worker to have woken: each loop is a shared job object, and a
// worker that wakes after its loop ended finds the job's counter exhausted and touches
// nothing of the caller's.  A worker that finishes a loop polls for the next one for a
// short while before it sleeps.
#pragma once

#include <atomic>
#include <condition_variable>
#include <functional>
#include <memory>
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
		// Runs `task` later on a background thread of its own, in submission order (used to
		// release large temporary structures without making the caller wait).
		void Later(std::function<void()> task);
		~WorkerPool();

	private:
		struct Job
		{
			const std::function<void(int)>* Body = nullptr;
			int Count = 0;
			std::atomic<int> Next{ 0 };
			std::atomic<int> Finished{ 0 };
		};

		WorkerPool();
		void Run();
		static void Drain(Job& job);

		std::vector<std::thread> Threads;
		std::mutex Busy;                    // held by the thread whose loop is running
		std::mutex M;                       // guards Current and sleeping on Wake
		std::condition_variable Wake;
		std::shared_ptr<Job> Current;
		std::atomic<uint64_t> Generation{ 0 };
		std::atomic<bool> Stop{ false };

		std::thread Background;             // started by the first Later call
		std::mutex LaterMutex;
		std::condition_variable LaterWake;
		std::vector<std::function<void()>> LaterTasks;
		bool LaterStop = false;
	};
}
