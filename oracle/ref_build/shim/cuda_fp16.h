#pragma once
/* Host-build stand-in for <cuda_fp16.h>.  The reference's FP16/WMMA path
 * (mode 0) is not emulated; the type only has to compile. */
struct half {
  float v;
  half() : v(0.f) {}
  template <class T> half(T t) : v((float)t) {}
};
