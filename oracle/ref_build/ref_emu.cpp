/* Thread-local launch coordinates for the host emulation (ref_emu.h). */
#include "ref_emu.h"

thread_local ref_uint3 threadIdx, blockIdx, blockDim, gridDim;
thread_local std::barrier<> *ref_emu_bar = nullptr;

void ref_emu_syncthreads(void) {
  if (ref_emu_bar) ref_emu_bar->arrive_and_wait();
}
