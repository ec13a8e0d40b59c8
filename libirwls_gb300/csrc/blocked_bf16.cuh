// blocked_bf16.cuh -- blocked bf16 layout of the precision form's SGMA
// operands, shared by the kernels that write them (dev_budget.cu: W;
// dev_tc.cu: Q) and the tcgen05 score kernel that streams them.
#pragma once
#include <stddef.h>

// Blocked bf16 layout of the precision form's Q (rows x ldq) and W (64 x
// ldq): for each 128-row tile (Q) and each block of 32 columns, the hi, mid
// and lo pieces of the FP32 values (hi = bf16(x), mid = bf16(x - hi), lo =
// bf16(x - hi - mid): together exactly x), each in the canonical K-major
// core-matrix order of a tcgen05 operand without swizzle (8 rows x 16 bytes
// per core matrix, core matrices 128 bytes apart along K and 512 bytes apart
// along rows). A score stage is thereby one contiguous 24 KB block of Q and
// one 12 KB block of W. Q takes ceil(rows / 128) * 128 * ldq * 6 bytes and W
// 64 * ldq * 6 bytes; kbn = ldq / 32 blocks per tile (ldq a multiple of 32).
constexpr int QB_NP = 3;                                // pieces per value
constexpr int QB_PIECE = 128 * 32, WB_PIECE = 64 * 32;  // elements per piece

__device__ __forceinline__ size_t qb_index(int i, int k, int kbn, int piece) {
    const int r = i & 127, c = k & 31;
    return (((size_t)(i >> 7) * kbn + (k >> 5)) * QB_NP + piece) * QB_PIECE + (r >> 3) * 256 + (c >> 3) * 64 +
           (r & 7) * 8 + (c & 7);
}

__device__ __forceinline__ size_t wb_index(int c_row, int k, int piece) {
    const int c = k & 31;
    return ((size_t)(k >> 5) * QB_NP + piece) * WB_PIECE + (c_row >> 3) * 256 + (c >> 3) * 64 + (c_row & 7) * 8 +
           (c & 7);
}

// The three pieces of x (each subtraction is exact, so hi + mid + lo == x).
__device__ __forceinline__ void bf16_pieces3(float x, __nv_bfloat16 p[3]) {
    p[0] = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p[0]);
    p[1] = __float2bfloat16_rn(r1);
    p[2] = __float2bfloat16_rn(r1 - __bfloat162float(p[1]));
}

// x from its pieces (exact).
__device__ __forceinline__ float bf16_join3(__nv_bfloat16 h, __nv_bfloat16 m, __nv_bfloat16 l) {
    return (__bfloat162float(h) + __bfloat162float(m)) + __bfloat162float(l);
}
