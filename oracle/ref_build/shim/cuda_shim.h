/*
 * cuda_shim.h — force-included when the reference's CUDA sources are compiled
 * as host C++ (oracle/ref_build/Makefile).  TEST INFRASTRUCTURE ONLY.
 *
 * Kernels become plain functions.  A launch is emulated by ref_emu.cpp: one
 * host thread per CUDA thread of a block, blocks one after another, and
 * __syncthreads() is a real barrier across the block's threads.  __shared__
 * variables become function-local statics, which all threads of the running
 * block share, as on the GPU.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__ static
#define __shared__ static

struct ref_uint3 { unsigned int x, y, z; };
extern thread_local ref_uint3 threadIdx, blockIdx, blockDim, gridDim;
void ref_emu_syncthreads(void);
static inline void __syncthreads(void) { ref_emu_syncthreads(); }

struct short2 { short x, y; };
struct ushort2 { unsigned short x, y; };
struct char4 { signed char x, y, z, w; };
struct uchar4 { unsigned char x, y, z, w; };
