// Device-side NTT plan layout shared by the translation units that run NTT kernels: the stage
// program and twiddle table a plan uploads (built by csrc/ntt.cu:build_plan), the specialised
// shapes of the two large field descriptors with their compiled-in schedules, and the register /
// shared-memory building blocks of ntt_fast.cuh.
#pragma once
#include "common.cuh"

namespace {

/// Division by an invariant divisor d (1 <= d < 2^32) with a multiply-high and shifts
/// (Granlund & Montgomery, "Division by invariant integers using multiplication", 1994, fig. 4.1).
struct FastDiv {
    uint32_t d, m, s1, s2;
};

struct DevStage {
    int32_t radix;      // 2 or 3
    int32_t stride;     // element stride of the factor's digit within the axis (suffix product)
    int32_t flen;       // factor length
    int32_t stage_len;  // length of one block in this stage
    int32_t tw_off;     // twiddle offset (pairs z,u): fwd r2: 1/block, fwd r3: 6/block, inv r2: 1, inv r3: 2
    int32_t zeta_off;   // inverse radix-3: offset of (zeta, zeta2)
    int32_t reduce_before;
    int32_t skip_ok;    // forward only
    int32_t last;       // last stage of the last factor (fwd: fusable reduction, inv: fused len^-1)
    int32_t span;       // (stage_len / radix) * stride: butterflies per group, distance of the legs
    FastDiv div_span;   // butterfly index -> (group, offset in group)
    FastDiv div_nblocks;  // group -> twiddle block (group mod flen / stage_len)
};

FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t l = 0;
    while (l < 32 && ((uint64_t)1 << l) < d) l++;
    f.m = (uint32_t)((((uint64_t)1 << 32) * ((((uint64_t)1) << l) - d)) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}

/// A pass of the kernel: either one stage through shared memory (kind 0, any radix), or k <= 3
/// consecutive radix-2 stages of one factor executed in registers (kind 1): each thread loads a
/// group of 2^k elements `span` apart, applies the k stages' butterflies to it in the
/// reference's order, and stores it back.
struct DevPass {
    int32_t kind;
    int32_t k;
    int32_t first;  // index of the pass's first stage in the (forward or inverse) program
    int32_t span;   // distance of consecutive group elements
    int32_t glen;   // extent of the block a group lies in (stage_len * stride)
    int32_t nb;     // blocks of that stage within the factor (twiddle block of a group)
    FastDiv div_span;
    FastDiv div_nb;
};

struct DevPlanHeader {
    int64_t n;
    int32_t len;
    int32_t nfwd;
    int32_t ninv;
    int32_t ntw;
    int32_t nfpass;
    int32_t nipass;
    int64_t one_z, one_u, invlen_z, invlen_u;
    DevStage fwd[HC_MAX_STAGES];
    DevStage inv[HC_MAX_STAGES];
    DevPass fpass[HC_MAX_STAGES];
    DevPass ipass[HC_MAX_STAGES];
    // followed by the twiddle table: ntw pairs (z, u)
};

struct PlanPtrs {
    const DevPlanHeader* p[HC_MAX_MODS];
};

}  // namespace

namespace {
#include "ntt_fast.cuh"

#define HC_SHAPE_GENERIC 0
#define HC_SHAPE_L3072 1   // dimension-3 line [2, 3, 8, 64]
#define HC_SHAPE_L12288 2  // dimension-3 line [3, 64, 64]
#define HC_SHAPE_C12 3     // dimension-2 column [4, 3]
#define HC_SHAPE_C4 4      // dimension-2 column [4]

__host__ __device__ constexpr int line_len(int shape) { return shape == HC_SHAPE_L3072 ? 3072 : 12288; }
__host__ __device__ constexpr int line_tile_words(int shape) { return line_len(shape) + line_len(shape) / 8; }

__device__ __forceinline__ fast::Ctx make_ctx(const DevPlanHeader* P, const int64_t* tw) {
    fast::Ctx c;
    c.n = P->n, c.one_z = P->one_z, c.one_u = P->one_u, c.il_z = P->invlen_z, c.il_u = P->invlen_u;
    c.tw = tw;
    return c;
}

/// The reduction / skip / fused-final schedule that the plans of the rings' primes have, per shape
/// and direction (bit s = the flag of stage s): field_36864 samples primes just below 2^57,
/// field_49152 primes just below 2^56.
struct SchedMasks {
    uint32_t fred, fskip, flast, ired, ilast;
};
__host__ __device__ constexpr SchedMasks fixed_masks(int shape) {
    return shape == HC_SHAPE_L3072    ? SchedMasks{0u, 0xFu, 1u << 10, 0x410u, 1u << 10}
           : shape == HC_SHAPE_L12288 ? SchedMasks{0u, 0x1Fu, 1u << 12, 0x1020u, 1u << 12}
           : shape == HC_SHAPE_C12    ? SchedMasks{0u, 0x7u, 1u << 2, 0u, 1u << 2}
           : shape == HC_SHAPE_C4     ? SchedMasks{0u, 0x3u, 1u << 1, 0u, 1u << 1}
                                      : SchedMasks{0u, 0u, 0u, 0u, 0u};
}
template <int SHAPE, bool INV>
using FixedSched = fast::FixSched<INV ? fixed_masks(SHAPE).ired : fixed_masks(SHAPE).fred,
                                  INV ? 0u : fixed_masks(SHAPE).fskip,
                                  INV ? fixed_masks(SHAPE).ilast : fixed_masks(SHAPE).flast>;

}  // namespace
