// Helpers of the tensor-core kernels whose operands are built in shared memory
// by producer warps (projections_tc.cu, the tensor-core Dmats in dmats.cu):
// the 128-byte swizzled K-major tile layout the UMMA descriptors read, the
// TF32 (hi, lo) split, and the producer barrier that ORs a flag.
#pragma once
#include "lelph_common.cuh"

// byte offset of the 16-byte chunk c of row r in a 128-byte swizzled K-major
// tile of 128-byte rows (8-row groups of 1024 bytes, chunk c ^ (r & 7))
__device__ __forceinline__ uint32_t tc_swz128(int r, int c)
{
    return (uint32_t)r * 128u + ((uint32_t)(c ^ (r & 7)) << 4);
}

// hi = rn_tf32(v), lo = rn_tf32(v - hi) of four values
__device__ __forceinline__ void tc_split4_tf32(float4 v, float4& h, float4& l)
{
    h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
    l = make_float4(tf32_rn(v.x - h.x), tf32_rn(v.y - h.y), tf32_rn(v.z - h.z), tf32_rn(v.w - h.w));
}

// barrier of the NTHR producer threads (named barrier 1) that also ORs a
// per-thread flag over them: every producer gets the same answer, so that the
// producers leave their loops together (a shared flag read after a plain
// barrier could differ between them when another role sets it meanwhile)
template <int NTHR>
__device__ __forceinline__ bool tc_producer_bar_any(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(NTHR)
        : "memory");
    return r != 0;
}
