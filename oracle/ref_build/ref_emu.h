/*
 * ref_emu.h — host emulation of CUDA launches for the reference's kernels.
 * TEST INFRASTRUCTURE ONLY (see cuda_shim.h).
 */
#pragma once
#include <barrier>
#include <thread>
#include <vector>

#include "shim/cuda_shim.h"

extern thread_local std::barrier<> *ref_emu_bar;

/* Runs fn() as grid x block CUDA threads.  Blocks run one after another.
 * With barrier=false the threads of a block run sequentially (valid for
 * kernels without __syncthreads); with barrier=true every thread of the block
 * is a host thread and __syncthreads() waits for all of them. */
template <class F>
void ref_launch(unsigned grid, unsigned block, bool barrier, F &&fn) {
  for (unsigned b = 0; b < grid; b++) {
    if (!barrier) {
      for (unsigned t = 0; t < block; t++) {
        gridDim = {grid, 1, 1};
        blockDim = {block, 1, 1};
        blockIdx = {b, 0, 0};
        threadIdx = {t, 0, 0};
        fn();
      }
    } else {
      std::barrier<> bar(block);
      std::vector<std::thread> th;
      th.reserve(block);
      for (unsigned t = 0; t < block; t++)
        th.emplace_back([&, t] {
          gridDim = {grid, 1, 1};
          blockDim = {block, 1, 1};
          blockIdx = {b, 0, 0};
          threadIdx = {t, 0, 0};
          ref_emu_bar = &bar;
          fn();
          ref_emu_bar = nullptr;
        });
      for (auto &x : th) x.join();
    }
  }
}
