#pragma once
/* Host-build stand-in for <mma.h>: WMMA declarations so that the reference's
 * tensor-core kernels compile.  They are never called from the host driver. */
#include "cuda_fp16.h"
namespace nvcuda {
namespace wmma {
struct matrix_a {};
struct matrix_b {};
struct accumulator {};
struct row_major {};
struct col_major {};
enum layout_t { mem_row_major, mem_col_major };
template <class Use, int M, int N, int K, class T, class Layout = void>
struct fragment { T x[1]; };
template <class F, class V> inline void fill_fragment(F &, V) {}
template <class F, class P> inline void load_matrix_sync(F &, const P *, unsigned) {}
template <class D, class A, class B, class C> inline void mma_sync(D &, const A &, const B &, const C &) {}
template <class P, class F> inline void store_matrix_sync(P *, const F &, unsigned, layout_t) {}
}  // namespace wmma
}  // namespace nvcuda
