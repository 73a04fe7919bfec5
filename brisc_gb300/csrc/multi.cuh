// Fused multi-solve launches (internal).
//
// A batch of independent IRLBA solves (per-subset PCAs) runs its Lanczos
// steps in lock step: each kernel of a step is ONE launch over every active
// solve. The launch takes a task list by value (a __grid_constant__ kernel
// parameter, up to kMaxTasks tasks): task i owns the CTAs [first[i],
// first[i+1]) of the grid, and each of those CTAs runs the single-solve
// kernel's body on task i's arguments with its block index and grid size
// taken relative to the task. A task's CTAs therefore compute exactly what
// the single-solve launch computes, in the same order, and a solve's results
// are bit-identical whether it runs alone or in a batch.
#pragma once

#include "common.cuh"

namespace bgpu {

constexpr uint32_t kMaxTasks = 64;

template <typename T>
struct TaskList {
  T t[kMaxTasks];
  uint32_t first[kMaxTasks + 1];  // first CTA of each task; first[count] = grid
  uint32_t count;

  // host: append a task that runs on `ctas` CTAs (a task with none is left
  // out: every listed task owns at least one CTA); callers add at most
  // kMaxTasks tasks (a larger batch is launched in chunks)
  void add(const T& task, uint32_t ctas) {
    if (ctas == 0) return;
    if (count == 0) first[0] = 0;
    t[count] = task;
    first[count + 1] = first[count] + ctas;
    ++count;
  }
  uint32_t grid() const { return count ? first[count] : 0u; }
};

template <typename T>
inline void task_list_init(TaskList<T>& L) {
  L.count = 0;
  L.first[0] = 0;
}

// The task owning CTA b: the largest i with first[i] <= b (every task owns
// at least one CTA, so the first[] prefix is strictly increasing).
__device__ __forceinline__ uint32_t task_of(const uint32_t* first, uint32_t count,
                                            uint32_t b) {
  uint32_t lo = 0, hi = count - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (first[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace bgpu
