/*
 * Minimal oneTBB stand-in used only to build the MSBG reference library as a
 * CPU oracle (oneTBB is not installed in this image).  It provides exactly the
 * TBB names the reference uses (src/thread.h:28, src/thread.h:287-330,
 * src/msbg.cpp:4571-4575, src/msbg2.cpp:48, src/thread.cpp:180-198) and runs
 * parallel_for on OpenMP threads, with the OpenMP thread number standing in for
 * the task-arena thread index that the reference uses to pick its per-thread
 * scratch (HaloBlockSet slot, ThrRunParallel locals).
 *
 * Test infrastructure only: nothing in the GPU product links this.
 */
#ifndef MSBG_ORACLE_TBB_SHIM_H
#define MSBG_ORACLE_TBB_SHIM_H

#include <algorithm>
#include <cstddef>
#include <omp.h>

namespace tbb {

template <typename Value>
class blocked_range {
 public:
  blocked_range(Value b, Value e) : b_(b), e_(e) {}
  Value begin() const { return b_; }
  Value end() const { return e_; }
  std::size_t size() const { return (std::size_t)(e_ - b_); }
  bool empty() const { return !(b_ < e_); }

 private:
  Value b_, e_;
};

/* Static chunks of 16 tasks per OpenMP iteration: the reference's per-task
 * work (one block) is uniform enough that a dynamic schedule is not needed,
 * and the thread index stays stable inside a chunk. */
template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &r, const Body &body) {
  const long long n = (long long)r.size();
  const long long chunk = 16;
  const long long nChunks = (n + chunk - 1) / chunk;
#pragma omp parallel for schedule(dynamic, 1)
  for (long long c = 0; c < nChunks; c++) {
    Value b = (Value)(r.begin() + c * chunk);
    Value e = (Value)std::min<long long>((long long)r.begin() + (c + 1) * chunk,
                                         (long long)r.end());
    body(blocked_range<Value>(b, e));
  }
}

template <typename It, typename Cmp>
void parallel_sort(It first, It last, const Cmp &cmp) {
  std::sort(first, last, cmp);
}

template <typename It>
void parallel_sort(It first, It last) {
  std::sort(first, last);
}

namespace this_task_arena {
inline int current_thread_index() { return omp_get_thread_num(); }
inline int max_concurrency() { return omp_get_max_threads(); }
}  // namespace this_task_arena

class task_scheduler_init {
 public:
  static int default_num_threads() { return omp_get_max_threads(); }
};

class global_control {
 public:
  enum parameter { max_allowed_parallelism, thread_stack_size };
  global_control(parameter p, std::size_t v) {
    if (p == max_allowed_parallelism && v > 0) omp_set_num_threads((int)v);
  }
};

}  // namespace tbb

#endif
