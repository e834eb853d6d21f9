// Lazy radix-2/3 group NTTs along dimension 2 or 3 of a ring-element tensor.
//
// The reference applies, per cyclic factor and per stage, Cooley-Tukey butterflies whose twiddle
// products are Barrett multiplications and whose sums stay unreduced; full reduction passes are
// inserted only where a data-independent worst-case bound says the next stage could overflow
// (cyclosubfield-dbfv/src/hal/ntt.rs:301-537, plan level :581-657). Because that schedule does
// not depend on the data, the host simulates it once per plan and stores a *stage program*
// (radix, geometry, reduce-before, twiddle-1 skip permission, fused final reduction/scaling)
// next to the twiddle constants in device memory. The kernel executes the program over a tile
// held in shared memory: a dimension-3 line (one CTA per line), or a block of dimension-2
// columns (one CTA per column block). Each butterfly performs exactly the reference's integer
// formula, so outputs are bit-identical; stages are not algebraically merged.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "ntt_plan.cuh"

namespace {

// ---------------------------------------------------------------- host-side constants
int64_t h_mul_mod(int64_t a, int64_t b, int64_t q) { return (int64_t)(((i128)a * (i128)b) % (i128)q); }
int64_t h_pow_mod(int64_t b, uint64_t e, int64_t q) {
    int64_t r = 1;
    b %= q;
    while (e) {
        if (e & 1) r = h_mul_mod(r, b, q);
        b = h_mul_mod(b, b, q);
        e >>= 1;
    }
    return r;
}
bool is_pow2(uint64_t x) { return x && !(x & (x - 1)); }
int64_t h_find_root(int64_t q, uint64_t n) {
    uint64_t p = is_pow2(n) ? 2 : 3;
    for (int64_t c = 2;; c++) {
        int64_t root = h_pow_mod(c, (uint64_t)((q - 1) / (int64_t)n), q);
        if (h_pow_mod(root, n / p, q) != 1) return root;
    }
}
/// BarrettMul::new (src/hal/ntt.rs:134-144): centred z, u = round(-z 2^64 / n).
void h_barrett(int64_t value, int64_t n, int64_t* z_out, int64_t* u_out) {
    int64_t z = value % n;
    if (2 * (i128)z > n) z -= n;
    else if (2 * (i128)z < -n) z += n;
    i128 a = -((i128)z << 64), b = n;
    i128 u = a >= 0 ? (a + b / 2) / b : -((-a + b / 2) / b);
    *z_out = z;
    *u_out = (int64_t)u;
}

struct HostPlan {
    DevPlanHeader h;
    std::vector<int64_t> tw;  // pairs
    void push(int64_t value) {
        int64_t z, u;
        h_barrett(value, h.n, &z, &u);
        tw.push_back(z);
        tw.push_back(u);
    }
    int32_t next_tw() const { return (int32_t)(tw.size() / 2); }
};

const u128 I64MAX = (u128)INT64_MAX;

}  // namespace

struct hc_ntt_plan_s {
    void* dev;        // DevPlanHeader + twiddles
    int64_t n;
    int32_t len;
    int32_t ntw;      // twiddle pairs
    int32_t shape;    // HC_SHAPE_*: factorisation with a specialised kernel
    bool fixed;       // the plan's schedule is the shape's compiled-in schedule
    size_t bytes;
};

// ---------------------------------------------------------------- device kernel
namespace {

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

/// Shared-memory slot of tile element i: for single lines (one vector) the low four index bits
/// are XOR-ed with the next four, so that groups of consecutive elements read by consecutive
/// threads fall into distinct banks; blocks of 16 stay in place, so the map is a permutation
/// whenever the line length is a multiple of 16.
__device__ __forceinline__ int sw(int i, bool on) { return on ? (i ^ ((i >> 4) & 15)) : i; }

/// Butterfly b of a stage -> position of its first leg (element index within the tile's
/// transform axis) and its twiddle block. Groups of `span` butterflies share a block; the legs of
/// a butterfly are `span` elements apart.
__device__ __forceinline__ int leg0(uint32_t bb, const DevStage& st, int* block) {
    uint32_t g = fdiv(bb, st.div_span);
    uint32_t off = bb - g * (uint32_t)st.span;
    uint32_t q = fdiv(g, st.div_nblocks);
    *block = (int)(g - q * st.div_nblocks.d);
    return (int)(g * (uint32_t)(st.stage_len * st.stride) + off);
}

struct Tile {
    int64_t* __restrict__ s;
    int len, logv;
    bool swz;
    __device__ __forceinline__ int64_t& at(int e, int v) const { return s[sw((e << logv) + v, swz)]; }
};

/// One forward stage (radix 2 or 3) over the tile in shared memory.
__device__ __forceinline__ void fwd_stage(const Tile& T, const DevStage st, const int64_t* __restrict__ tw,
                                          int64_t n, int64_t one_z, int64_t one_u, bool reduce_output) {
    const int radix = st.radix;
    const bool fuse = st.last && reduce_output;
    const int nbf = (T.len / radix) << T.logv;
    const int vmask = (1 << T.logv) - 1;
    for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
        int block;
        const int e = leg0((uint32_t)(b >> T.logv), st, &block), v = b & vmask;
        int64_t& x = T.at(e, v);
        int64_t& y = T.at(e + st.span, v);
        if (radix == 2) {
            int64_t z = tw[2 * (st.tw_off + block)], u = tw[2 * (st.tw_off + block) + 1];
            bool skip = st.skip_ok && z == 1;
            int64_t a = x, yv = y;
            if (st.reduce_before) {  // the reference's reduction pass, applied as the operands are read
                a = bmul1(one_u, a, n);
                yv = bmul1(one_u, yv, n);
            }
            int64_t t = skip ? yv : bmul(z, u, yv, n);
            int64_t o0 = wadd(a, t), o1 = wsub(a, t);
            if (fuse) {
                o0 = bmul1(one_u, o0, n);
                o1 = bmul1(one_u, o1, n);
            }
            x = o0;
            y = o1;
        } else {
            int64_t& zr = T.at(e + 2 * st.span, v);
            const int64_t* w = tw + 2 * (st.tw_off + 6 * block);
            bool skip = st.skip_ok && w[0] == 1;
            int64_t a = x, bv = y, c = zr;
            if (st.reduce_before) {
                a = bmul1(one_u, a, n);
                bv = bmul1(one_u, bv, n);
                c = bmul1(one_u, c, n);
            }
            int64_t t_b = skip ? bv : bmul(w[0], w[1], bv, n);
            int64_t t_bz = bmul(w[2], w[3], bv, n);
            int64_t t_bzz = bmul(w[4], w[5], bv, n);
            int64_t t_c = skip ? c : bmul(w[6], w[7], c, n);
            int64_t t_cz = bmul(w[8], w[9], c, n);
            int64_t t_czz = bmul(w[10], w[11], c, n);
            int64_t o0 = wadd(wadd(a, t_b), t_c), o1 = wadd(wadd(a, t_bz), t_czz), o2 = wadd(wadd(a, t_bzz), t_cz);
            if (fuse) {
                o0 = bmul1(one_u, o0, n);
                o1 = bmul1(one_u, o1, n);
                o2 = bmul1(one_u, o2, n);
            }
            x = o0;
            y = o1;
            zr = o2;
        }
    }
}

/// One inverse stage (radix 2 or 3) over the tile in shared memory.
__device__ __forceinline__ void inv_stage(const Tile& T, const DevStage st, const int64_t* __restrict__ tw,
                                          int64_t n, int64_t il_z, int64_t il_u, int64_t one_z, int64_t one_u) {
    const int radix = st.radix;
    const bool fused = st.last;
    const int nbf = (T.len / radix) << T.logv;
    const int vmask = (1 << T.logv) - 1;
    for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
        int block;
        const int e = leg0((uint32_t)(b >> T.logv), st, &block), v = b & vmask;
        int64_t& x = T.at(e, v);
        int64_t& y = T.at(e + st.span, v);
        if (radix == 2) {
            int64_t yz, yu;
            if (fused) {
                yz = il_z;
                yu = il_u;
            } else {
                yz = tw[2 * (st.tw_off + block)];
                yu = tw[2 * (st.tw_off + block) + 1];
            }
            bool skip = !fused && yz == 1;
            int64_t y0 = x, y1 = y;
            if (st.reduce_before) {
                y0 = bmul1(one_u, y0, n);
                y1 = bmul1(one_u, y1, n);
            }
            int64_t sum = wadd(y0, y1), dif = wsub(y0, y1);
            x = fused ? bmul(yz, yu, sum, n) : sum;
            y = skip ? dif : bmul(yz, yu, dif, n);
        } else {
            int64_t& zr = T.at(e + 2 * st.span, v);
            int64_t yz, yu, zz, zu;
            if (fused) {
                yz = zz = il_z;
                yu = zu = il_u;
            } else {
                const int64_t* w = tw + 2 * (st.tw_off + 2 * block);
                yz = w[0], yu = w[1], zz = w[2], zu = w[3];
            }
            bool skip = !fused && yz == 1;
            const int64_t* zt = tw + 2 * st.zeta_off;
            int64_t y0 = x, y1 = y, y2 = zr;
            if (st.reduce_before) {
                y0 = bmul1(one_u, y0, n);
                y1 = bmul1(one_u, y1, n);
                y2 = bmul1(one_u, y2, n);
            }
            int64_t y1z = bmul(zt[0], zt[1], y1, n), y1zz = bmul(zt[2], zt[3], y1, n);
            int64_t y2z = bmul(zt[0], zt[1], y2, n), y2zz = bmul(zt[2], zt[3], y2, n);
            int64_t s0 = wadd(wadd(y0, y1), y2);
            int64_t sy = wadd(wadd(y0, y1zz), y2z), sz = wadd(wadd(y0, y1z), y2zz);
            x = fused ? bmul(yz, yu, s0, n) : s0;
            y = skip ? sy : bmul(yz, yu, sy, n);
            zr = skip ? sz : bmul(zz, zu, sz, n);
        }
    }
}

/// K consecutive forward radix-2 stages of one factor in registers. Group element m lies at
/// g * glen + o + m * span; at the q-th stage of the pass the butterflies pair m with
/// m + 2^(K-1-q) and use the twiddle of block block0 * 2^q + (m >> (K-q)).
template <int K>
__device__ __forceinline__ void fwd_pass_r2(const Tile& T, const DevPass ps, const DevStage* sts,
                                            const int64_t* __restrict__ tw, int64_t n, int64_t one_z, int64_t one_u,
                                            bool reduce_output) {
    constexpr int M = 1 << K;
    // the stage parameters, read once into registers
    int tw_off[K];
    bool red[K], skip_ok[K], fuse[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        const DevStage& st = sts[ps.first + q];
        tw_off[q] = st.tw_off;
        red[q] = st.reduce_before;
        skip_ok[q] = st.skip_ok;
        fuse[q] = st.last && reduce_output;
    }
    const int ng = (T.len >> K) << T.logv;
    const int vmask = (1 << T.logv) - 1;
    for (int gi = threadIdx.x; gi < ng; gi += blockDim.x) {
        const int v = gi & vmask;
        const uint32_t gg = (uint32_t)(gi >> T.logv);
        const uint32_t g = fdiv(gg, ps.div_span);
        const int o = (int)(gg - g * (uint32_t)ps.span);
        const int block0 = (int)(g - fdiv(g, ps.div_nb) * (uint32_t)ps.nb);
        const int base = (int)g * ps.glen + o;
        int64_t x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = T.at(base + m * ps.span, v);
#pragma unroll
        for (int q = 0; q < K; q++) {
            if (red[q]) {
#pragma unroll
                for (int m = 0; m < M; m++) x[m] = bmul1(one_u, x[m], n);
            }
            const int half = M >> (q + 1);
#pragma unroll
            for (int j = 0; j < M / 2; j++) {
                const int m1 = ((j / half) * 2 * half) + (j % half), m2 = m1 + half;
                const int tb = block0 * (1 << q) + (m1 >> (K - q));
                const int64_t z = tw[2 * (tw_off[q] + tb)], u = tw[2 * (tw_off[q] + tb) + 1];
                const bool skip = skip_ok[q] && z == 1;
                const int64_t a = x[m1];
                const int64_t t = skip ? x[m2] : bmul(z, u, x[m2], n);
                int64_t o0 = wadd(a, t), o1 = wsub(a, t);
                if (fuse[q]) {
                    o0 = bmul1(one_u, o0, n);
                    o1 = bmul1(one_u, o1, n);
                }
                x[m1] = o0;
                x[m2] = o1;
            }
        }
#pragma unroll
        for (int m = 0; m < M; m++) T.at(base + m * ps.span, v) = x[m];
    }
}

/// K consecutive inverse radix-2 stages (stage lengths growing) in registers: at the q-th stage
/// of the pass the butterflies pair m with m + 2^q and use the twiddle of block
/// blockK * 2^(K-1-q) + (m >> (q+1)), blockK being the group's block at the pass's last stage.
template <int K>
__device__ __forceinline__ void inv_pass_r2(const Tile& T, const DevPass ps, const DevStage* sts,
                                            const int64_t* __restrict__ tw, int64_t n, int64_t il_z, int64_t il_u,
                                            int64_t one_z, int64_t one_u) {
    constexpr int M = 1 << K;
    int tw_off[K];
    bool red[K], fused[K];
#pragma unroll
    for (int q = 0; q < K; q++) {
        const DevStage& st = sts[ps.first + q];
        tw_off[q] = st.tw_off;
        red[q] = st.reduce_before;
        fused[q] = st.last;
    }
    const int ng = (T.len >> K) << T.logv;
    const int vmask = (1 << T.logv) - 1;
    for (int gi = threadIdx.x; gi < ng; gi += blockDim.x) {
        const int v = gi & vmask;
        const uint32_t gg = (uint32_t)(gi >> T.logv);
        const uint32_t g = fdiv(gg, ps.div_span);
        const int o = (int)(gg - g * (uint32_t)ps.span);
        const int blockK = (int)(g - fdiv(g, ps.div_nb) * (uint32_t)ps.nb);
        const int base = (int)g * ps.glen + o;
        int64_t x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = T.at(base + m * ps.span, v);
#pragma unroll
        for (int q = 0; q < K; q++) {
            if (red[q]) {
#pragma unroll
                for (int m = 0; m < M; m++) x[m] = bmul1(one_u, x[m], n);
            }
            const int dist = 1 << q;
#pragma unroll
            for (int j = 0; j < M / 2; j++) {
                const int m1 = ((j >> q) << (q + 1)) | (j & (dist - 1)), m2 = m1 + dist;
                const int tb = blockK * (1 << (K - 1 - q)) + (m1 >> (q + 1));
                int64_t yz, yu;
                if (fused[q]) {
                    yz = il_z;
                    yu = il_u;
                } else {
                    yz = tw[2 * (tw_off[q] + tb)];
                    yu = tw[2 * (tw_off[q] + tb) + 1];
                }
                const bool skip = !fused[q] && yz == 1;
                const int64_t y0 = x[m1], y1 = x[m2];
                const int64_t sum = wadd(y0, y1), dif = wsub(y0, y1);
                x[m1] = fused[q] ? bmul(yz, yu, sum, n) : sum;
                x[m2] = skip ? dif : bmul(yz, yu, dif, n);
            }
        }
#pragma unroll
        for (int m = 0; m < M; m++) T.at(base + m * ps.span, v) = x[m];
    }
}

#ifndef HC_NTT_MIN_BLOCKS
#define HC_NTT_MIN_BLOCKS 3  // resident CTAs per SM the register allocation must allow
#endif

/// Where one tile lives in global memory and where its Montgomery multiplier (modes 2 and 3)
/// comes from: element (e, v) of the tile is g[e * ge + v] and is multiplied by
/// mulp[e * me + v * mv] modulo (mn, mi).
struct TileIO {
    int64_t* g;
    int64_t ge;
    int64_t ncol;  // valid columns of the tile (a dimension-2 block at the end of the axis)
    const int64_t* mulp;
    int64_t me, mv;
    int64_t mn, mi;
};

/// One tile transformed by plan P, twiddles `tw` already staged. mode 0: forward (reduced),
/// 1: inverse, 2: forward unreduced + Montgomery multiplication, 3: inverse + Montgomery
/// multiplication. With `use_smem` the tile is copied to `s` (len x 2^logv elements) and back;
/// otherwise (single lines too long for shared memory) it is worked on in place in global memory.
/// Ends with a block barrier, so the caller may reuse the shared memory at once.
__device__ __forceinline__ void tile_run(const DevPlanHeader* __restrict__ P, const int64_t* __restrict__ tw,
                                         int64_t* s, int len, int logv, bool use_smem, int mode,
                                         const TileIO& io) {
    const int V = 1 << logv, vmask = V - 1;
    const int64_t n = P->n;
    const int total = len * V;
    Tile T{use_smem ? s : io.g, len, logv, use_smem && logv == 0 && (len & 15) == 0};
    if (use_smem) {
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            int e = idx >> logv, v = idx & vmask;
            T.at(e, v) = v < io.ncol ? io.g[e * io.ge + v] : 0;
        }
    }
    __syncthreads();
    const bool inverse = mode & 1;
    const int npass = inverse ? P->nipass : P->nfpass;
    const int64_t one_z = P->one_z, one_u = P->one_u, il_z = P->invlen_z, il_u = P->invlen_u;
    for (int pi = 0; pi < npass; pi++) {
        const DevPass ps = inverse ? P->ipass[pi] : P->fpass[pi];
        if (ps.kind == 0) {
            if (inverse) inv_stage(T, P->inv[ps.first], tw, n, il_z, il_u, one_z, one_u);
            else fwd_stage(T, P->fwd[ps.first], tw, n, one_z, one_u, mode == 0);
        } else if (inverse) {
            if (ps.k == 3) inv_pass_r2<3>(T, ps, P->inv, tw, n, il_z, il_u, one_z, one_u);
            else if (ps.k == 2) inv_pass_r2<2>(T, ps, P->inv, tw, n, il_z, il_u, one_z, one_u);
            else inv_pass_r2<1>(T, ps, P->inv, tw, n, il_z, il_u, one_z, one_u);
        } else {
            if (ps.k == 3) fwd_pass_r2<3>(T, ps, P->fwd, tw, n, one_z, one_u, mode == 0);
            else if (ps.k == 2) fwd_pass_r2<2>(T, ps, P->fwd, tw, n, one_z, one_u, mode == 0);
            else fwd_pass_r2<1>(T, ps, P->fwd, tw, n, one_z, one_u, mode == 0);
        }
        __syncthreads();
    }
    // plans without factors (length 1): the inverse scales by 1^-1, the reduced forward
    // reduces; an unreduced forward leaves the data unchanged
    if (npass == 0 && (mode == 0 || inverse)) {
        int64_t fz = inverse ? P->invlen_z : P->one_z, fu = inverse ? P->invlen_u : P->one_u;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            int e = idx >> logv, v = idx & vmask;
            T.at(e, v) = bmul(fz, fu, T.at(e, v), n);
        }
        __syncthreads();
    }
    if (mode & 2) {
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            int e = idx >> logv, v = idx & vmask;
            if (v >= io.ncol) continue;
            T.at(e, v) = mul_mont(T.at(e, v), io.mulp[e * io.me + v * io.mv], io.mn, io.mi);
        }
        __syncthreads();
    }
    if (use_smem) {
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            int e = idx >> logv, v = idx & vmask;
            if (v < io.ncol) io.g[e * io.ge + v] = T.at(e, v);
        }
    }
    __syncthreads();
}

/// Copies the twiddle table of plan P to shared memory (no barrier).
__device__ __forceinline__ void stage_twiddles(const DevPlanHeader* P, int64_t* dst) {
    const int64_t* twg = reinterpret_cast<const int64_t*>(P + 1);
    for (int idx = threadIdx.x; idx < 2 * P->ntw; idx += blockDim.x) dst[idx] = twg[idx];
}

}  // namespace

namespace {

/// One specialised line g of plan P through the CTA's shared-memory line buffer s; FIX: the plan
/// has the fixed schedule.
template <int SHAPE, int MODE, bool FIX>
__device__ __forceinline__ void run_line(const DevPlanHeader* P, const fast::Ctx& c, int64_t* s, int64_t* g,
                                         const int64_t* mulp, int64_t me, int64_t mn, int64_t mi) {
    const DevStage* st = (MODE & 1) ? P->inv : P->fwd;
    if constexpr (FIX) {
        const FixedSched<SHAPE, (MODE & 1) != 0> sch{st};
        if constexpr (SHAPE == HC_SHAPE_L3072) fast::line3072<MODE>(sch, c, s, g, mulp, me, mn, mi);
        else fast::line12288<MODE>(sch, c, s, g, mulp, me, mn, mi);
    } else {
        const fast::DynSched sch{st};
        if constexpr (SHAPE == HC_SHAPE_L3072) fast::line3072<MODE>(sch, c, s, g, mulp, me, mn, mi);
        else fast::line12288<MODE>(sch, c, s, g, mulp, me, mn, mi);
    }
}

/// Specialised dimension-3 NTT: one line (i, j, k) per CTA.
template <int SHAPE, int MODE, bool FIX, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) ntt_line_kernel(KView t, PlanPtrs plans, KView mul, KMods mods) {
    extern __shared__ int64_t smem[];
    const int64_t tile = blockIdx.x;
    const int64_t k = tile % t.n2, r = tile / t.n2;
    const int64_t j = r % t.n1, i = r / t.n1;
    const DevPlanHeader* P = plans.p[j];
    // twiddles read from the plan in global memory (L1-cached): shared memory holds only the line
    const fast::Ctx c = make_ctx(P, reinterpret_cast<const int64_t*>(P + 1));
    int64_t* g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + k * t.s2;
    const int64_t* mulp = nullptr;
    int64_t me = 0, mn = 0, mi = 0;
    if (MODE & 2) {
        mulp = kat<int64_t>(mul, i, j, k, 0);
        me = mul.b3 ? 0 : 1;
        mn = mods.n[j], mi = mods.ninv[j];
    }
    run_line<SHAPE, MODE, FIX>(P, c, smem, g, mulp, me, mn, mi);
}

/// [3, 64, 64] lines along dimension 3 as 3-CTA clusters: CTA `blk` of a cluster computes block
/// blk (4096 residues) of one line.
static_assert(sizeof(DevPlanHeader) % 16 == 0, "plan twiddle table must be 16-byte aligned");
template <int MODE, bool FIX>
__global__ void __cluster_dims__(3, 1, 1) __launch_bounds__(128, 6)
    ntt_line3_kernel(KView t, PlanPtrs plans, KView mul, KMods mods) {
    extern __shared__ int64_t smem[];
    const int64_t tile = blockIdx.x / 3;
    const int blk = (int)(blockIdx.x % 3);
    const int64_t k = tile % t.n2, r = tile / t.n2;
    const int64_t j = r % t.n1, i = r / t.n1;
    const DevPlanHeader* P = plans.p[j];
    // twiddles read from the plan in global memory (L1-cached): the CTA's shared memory holds only
    // its 4096-residue block, so that six CTAs fit on an SM
    const fast::Ctx c = make_ctx(P, reinterpret_cast<const int64_t*>(P + 1));
    int64_t* g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + k * t.s2;
    const int64_t* mulp = nullptr;
    int64_t me = 0, mn = 0, mi = 0;
    if (MODE & 2) {
        mulp = kat<int64_t>(mul, i, j, k, 0);
        me = mul.b3 ? 0 : 1;
        mn = mods.n[j], mi = mods.ninv[j];
    }
    auto csync = [] { cooperative_groups::this_cluster().sync(); };
    const DevStage* st = (MODE & 1) ? P->inv : P->fwd;
    if constexpr (FIX) {
        const FixedSched<HC_SHAPE_L12288, (MODE & 1) != 0> sch{st};
        fast::line12288_block<MODE>(sch, c, smem, g, blk, mulp, me, mn, mi, csync);
    } else {
        const fast::DynSched sch{st};
        fast::line12288_block<MODE>(sch, c, smem, g, blk, mulp, me, mn, mi, csync);
    }
}

/// One specialised column g[0], g[ge], ... of shape SHAPE transformed in registers; it is read
/// from gs[0], gs[gse], ... (g itself for an in-place call).
template <int SHAPE, int MODE, bool FIX>
__device__ __forceinline__ void run_column(const DevPlanHeader* P, const fast::Ctx& c, int64_t* g, int64_t ge,
                                           const int64_t* gs, int64_t gse, const int64_t* mulp, int64_t mstride,
                                           int64_t mn, int64_t mi) {
    constexpr bool inv = MODE & 1;
    const DevStage* st = inv ? P->inv : P->fwd;
    constexpr int NST = SHAPE == HC_SHAPE_C12 ? 3 : 2;
    fast::SF f[NST];
    if constexpr (FIX) {
        const FixedSched<SHAPE, inv> sch{st};
#pragma unroll
        for (int q = 0; q < NST; q++) f[q] = fast::sflags(sch, q);
    } else {
        const fast::DynSched sch{st};
#pragma unroll
        for (int q = 0; q < NST; q++) f[q] = fast::sflags(sch, q);
    }
    if constexpr (SHAPE == HC_SHAPE_C12) {
        int64_t x[4][3];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) x[a][b] = gs[(3 * a + b) * gse];
        fast::col12(c, f, inv, MODE == 0, x);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                int64_t v = x[a][b];
                if (MODE & 2) v = mul_mont(v, mulp[(3 * a + b) * mstride], mn, mi);
                g[(3 * a + b) * ge] = v;
            }
    } else {
        int64_t x[4];
#pragma unroll
        for (int a = 0; a < 4; a++) x[a] = gs[a * gse];
        fast::col4(c, f, inv, MODE == 0, x);
#pragma unroll
        for (int a = 0; a < 4; a++) {
            int64_t v = x[a];
            if (MODE & 2) v = mul_mont(v, mulp[a * mstride], mn, mi);
            g[a * ge] = v;
        }
    }
}

#define HC_COL_THREADS 256
#ifndef HC_L3072_MIN_BLOCKS
#define HC_L3072_MIN_BLOCKS 8  // resident CTAs per SM the 3072-residue line kernel's registers must allow (8 fit its shared memory)
#endif
#ifndef HC_COL12_MIN_BLOCKS
#define HC_COL12_MIN_BLOCKS 4  // resident CTAs per SM the [4, 3] column kernel's registers must allow
#endif
#define HC_COL_TW 128  // twiddle words a column plan may have (checked at dispatch)

/// Specialised dimension-2 NTT: one thread per column (i, j, l), CTAs over (i, j, column block).
template <int SHAPE, int MODE, bool FIX>
__global__ void __launch_bounds__(HC_COL_THREADS, SHAPE == HC_SHAPE_C12 ? HC_COL12_MIN_BLOCKS : 4) ntt_col_kernel(KView t, PlanPtrs plans, KView mul, KMods mods,
                                                                    int ncb, KView src) {
    __shared__ __align__(16) int64_t tws[HC_COL_TW];
    // tiles last to first: a transform's column pass follows a line pass (or the input's producer)
    // that wrote the tensor first to last, so the CTAs scheduled first read what is still in L2,
    // and the next line pass, first to last, starts on what this pass wrote last
    const int64_t tile = gridDim.x - 1 - blockIdx.x;
    const int64_t cb = tile % ncb, r = tile / ncb;
    const int64_t j = r % t.n1, i = r / t.n1;
    const DevPlanHeader* P = plans.p[j];
    stage_twiddles(P, tws);
    __syncthreads();
    const int64_t l = cb * HC_COL_THREADS + threadIdx.x;
    if (l >= t.n3) return;
    const fast::Ctx c = make_ctx(P, tws);
    int64_t* g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + l;
    const int64_t* mulp = nullptr;
    int64_t ms = 0, mn = 0, mi = 0;
    if (MODE & 2) {
        mulp = kat<int64_t>(mul, i, j, 0, l);
        ms = mul.s2;
        mn = mods.n[j], mi = mods.ninv[j];
    }
    // out of place (src.p set): the column is read from src, written to t
    const int64_t* gs = src.p ? reinterpret_cast<const int64_t*>(src.p) + i * src.s0 + j * src.s1 + l : g;
    run_column<SHAPE, MODE, FIX>(P, c, g, t.s2, gs, src.p ? src.s2 : t.s2, mulp, ms, mn, mi);
}

/// Host: launches the specialised kernel of (shape, mode, fixed schedule).
template <int SHAPE, int MODE, bool FIX>
hc_status launch_special(hc_context ctx, const KView& t, const PlanPtrs& pp, const KView& mul, const KMods& mods,
                         size_t smem, int64_t tiles, int ncb, const KView& src) {
    if constexpr (SHAPE == HC_SHAPE_L12288) {
        // one 3-CTA cluster per line: padded 4096-residue block + twiddles per CTA
        const size_t smem3 = 4608 * 8;
        auto kern = ntt_line3_kernel<MODE, FIX>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem3);
        if (e != cudaSuccess) return hc::cuda_check(e, "ntt smem attribute");
        if (tiles * 3 > 0x7fffffff) return hc::fail(HC_ERR_UNSUPPORTED, "too many NTT lines in one call");
        kern<<<(unsigned)(tiles * 3), 128, smem3, hc::stream_of(ctx)>>>(t, pp, mul, mods);
    } else if constexpr (SHAPE == HC_SHAPE_L3072) {
        constexpr int TH = SHAPE == HC_SHAPE_L3072 ? 128 : 256, MB = SHAPE == HC_SHAPE_L3072 ? HC_L3072_MIN_BLOCKS : 2;
        auto kern = ntt_line_kernel<SHAPE, MODE, FIX, TH, MB>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return hc::cuda_check(e, "ntt smem attribute");
        kern<<<(unsigned)tiles, TH, smem, hc::stream_of(ctx)>>>(t, pp, mul, mods);
    } else {
        ntt_col_kernel<SHAPE, MODE, FIX><<<(unsigned)tiles, HC_COL_THREADS, 0, hc::stream_of(ctx)>>>(t, pp, mul, mods, ncb,
                                                                                                   src);
    }
    hc::count_launch(ctx);
    return hc::cuda_check(cudaGetLastError(), "ntt kernel launch");
}

template <int SHAPE>
hc_status launch_special_mode(hc_context ctx, int mode, bool fix, const KView& t, const PlanPtrs& pp, const KView& mul,
                              const KMods& mods, size_t smem, int64_t tiles, int ncb, const KView& src = KView()) {
    if (fix) {
        if (mode == 0) return launch_special<SHAPE, 0, true>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
        if (mode == 1) return launch_special<SHAPE, 1, true>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
        if (mode == 2) return launch_special<SHAPE, 2, true>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
        return launch_special<SHAPE, 3, true>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
    }
    if (mode == 0) return launch_special<SHAPE, 0, false>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
    if (mode == 1) return launch_special<SHAPE, 1, false>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
    if (mode == 2) return launch_special<SHAPE, 2, false>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
    return launch_special<SHAPE, 3, false>(ctx, t, pp, mul, mods, smem, tiles, ncb, src);
}

/// mode 0: forward (reduced), 1: inverse, 2: forward unreduced + Montgomery multiplication by `mul`.
/// dim 3: tile = line (i, j, k), element e at l = e.  dim 2: tile = (i, j, column block),
/// element (e, v) at k = e, l = cb * V + v.
__global__ void __launch_bounds__(256, HC_NTT_MIN_BLOCKS) ntt_tile_kernel(KView t, PlanPtrs plans, int dim, int mode, KView mul,
                                                       KMods mods, int logv, int ntile2, int use_smem) {
    extern __shared__ int64_t smem[];
    const int V = 1 << logv;
    const int len = dim == 3 ? (int)t.n3 : (int)t.n2;
    int64_t tile = blockIdx.x;
    int64_t i, j, k = 0, cb = 0;
    if (dim == 3) {
        k = tile % t.n2;
        int64_t r = tile / t.n2;
        j = r % t.n1;
        i = r / t.n1;
    } else {
        cb = tile % ntile2;
        int64_t r = tile / ntile2;
        j = r % t.n1;
        i = r / t.n1;
    }
    const DevPlanHeader* P = plans.p[j];
    // the plan's twiddle constants are staged in shared memory, behind the tile
    int64_t* tws = smem + (use_smem ? (size_t)len * V : 0);
    stage_twiddles(P, tws);
    TileIO io;
    io.g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + (dim == 3 ? k * t.s2 : cb * V);
    io.ge = dim == 3 ? 1 : t.s2;
    io.ncol = dim == 3 ? 1 : t.n3 - cb * V;
    io.mulp = nullptr, io.me = io.mv = 0, io.mn = io.mi = 0;
    if (mode & 2) {
        io.mulp = kat<int64_t>(mul, i, j, dim == 3 ? k : 0, dim == 3 ? 0 : cb * V);
        io.me = dim == 3 ? (mul.b3 ? 0 : 1) : mul.s2;
        io.mv = dim == 3 ? 0 : (mul.b3 ? 0 : 1);
        io.mn = mods.n[j], io.mi = mods.ninv[j];
    }
    tile_run(P, tws, smem, len, logv, use_smem, mode, io);
}

/// One pass of a batched transform over a whole slab: its deg_L' lines (dimension 3) or its
/// column blocks of 2^logv columns (dimension 2). Modes as tile_run; `mulrow` is the CRT kernel
/// row of the pass (modes 2 and 3 along dimension 2, mode 2 along dimension 3), while mode 3
/// along dimension 3 multiplies by the slab's operand.
template <bool GENERIC, int CLS>
__device__ __forceinline__ void slab_pass(const CrtSlab& S, const DevPlanHeader* P, const int64_t* tw, int64_t* s,
                                          int dim, int mode, const int64_t* mulrow, int logv) {
    // specialised kernels for slabs whose plans have the fixed schedule (bit 16: dimension-3
    // plan, bit 17: dimension-2 plan), the generic tile programme otherwise
    const int shape = dim == 3 ? (S.shapes & 0xff) : ((S.shapes >> 8) & 0xff);
    const bool fix = (S.shapes >> (dim == 3 ? 16 : 17)) & 1;
    if (fix && dim == 3 && (shape == HC_SHAPE_L3072 || shape == HC_SHAPE_L12288)) {
        const fast::Ctx c = make_ctx(P, tw);
        for (int k = 0; k < S.dl; k++) {
            int64_t* g = S.data + k * S.s2;
            const int64_t* mulp = mode == 3 ? S.op + k * S.op_s2 : mulrow;
            if (CLS != 2 && (CLS == 1 || shape == HC_SHAPE_L3072)) {
                if (mode == 2) run_line<HC_SHAPE_L3072, 2, true>(P, c, s, g, mulp, 1, S.n, S.ninv);
                else if (mode == 3) run_line<HC_SHAPE_L3072, 3, true>(P, c, s, g, mulp, 1, S.n, S.ninv);
                else run_line<HC_SHAPE_L3072, 1, true>(P, c, s, g, mulp, 1, S.n, S.ninv);
            } else if (CLS != 1) {
                // one 4096-residue block in shared memory at a time (crt_slab_tile_words)
                if (mode & 1) {  // modes 1 (inverse) and 3 (inverse, then the operand product)
                    const FixedSched<HC_SHAPE_L12288, true> sch{P->inv};
                    if (mode == 3) fast::line12288_seq<3>(sch, c, s, g, mulp, 1, S.n, S.ninv);
                    else fast::line12288_seq<1>(sch, c, s, g, mulp, 1, S.n, S.ninv);
                } else {  // mode 2: forward, then the kernel product
                    const FixedSched<HC_SHAPE_L12288, false> sch{P->fwd};
                    fast::line12288_seq<2>(sch, c, s, g, mulp, 1, S.n, S.ninv);
                }
            }
            __syncthreads();
        }
        return;
    }
    if (fix && dim == 2 && (shape == HC_SHAPE_C12 || shape == HC_SHAPE_C4)) {
        const fast::Ctx c = make_ctx(P, tw);
        for (int l = threadIdx.x; l < S.dk; l += blockDim.x) {
            if (CLS != 2 && (CLS == 1 || shape == HC_SHAPE_C12)) {
                if (mode == 2) run_column<HC_SHAPE_C12, 2, true>(P, c, S.data + l, S.s2, S.data + l, S.s2, mulrow, 1, S.n,
                                                             S.ninv);
                else run_column<HC_SHAPE_C12, 1, true>(P, c, S.data + l, S.s2, S.data + l, S.s2, mulrow, 1, S.n,
                                                             S.ninv);
            } else if (CLS != 1) {
                if (mode == 2) run_column<HC_SHAPE_C4, 2, true>(P, c, S.data + l, S.s2, S.data + l, S.s2, mulrow, 1, S.n,
                                                             S.ninv);
                else run_column<HC_SHAPE_C4, 1, true>(P, c, S.data + l, S.s2, S.data + l, S.s2, mulrow, 1, S.n,
                                                             S.ninv);
            }
        }
        __syncthreads();
        return;
    }
    if constexpr (!GENERIC) return;  // the launcher sends only specialised slabs to this form
    TileIO io;
    io.mn = S.n, io.mi = S.ninv;
    io.me = 1, io.mv = 0;
    if (dim == 3) {
        io.ge = 1, io.ncol = 1;
        for (int k = 0; k < S.dl; k++) {
            io.g = S.data + k * S.s2;
            io.mulp = mode == 3 ? S.op + k * S.op_s2 : mulrow;
            tile_run(P, tw, s, S.dk, 0, true, mode, io);
        }
    } else {
        const int V = 1 << logv;
        io.ge = S.s2;
        io.mulp = mulrow;
        for (int c0 = 0; c0 < S.dk; c0 += V) {
            io.g = S.data + c0;
            io.ncol = S.dk - c0 < V ? S.dk - c0 : V;
            tile_run(P, tw, s, S.dl, logv, true, mode, io);
        }
    }
}

/// Persistent batched CRT transforms: every CTA takes the next slab from `counter` and runs the
/// slab's whole operation (period -> CRT, Montgomery product with the operand, CRT -> period, as
/// its `ops` say) before taking another. Slabs of different fields and RNS lengths mix freely;
/// the passes are the HAL transforms' passes in the same order (src/ring.rs:1118-1161), the
/// operand product fused into the epilogue of the forward transform's last pass.
/// GENERIC = false: every slab has the specialised line and column shapes with compiled-in
/// schedules (both large fields' rings), so the generic tile programme is left out; MINB: the CTAs
/// of MAXT threads per SM the register allocation must allow (256 threads: 2 -> 128 registers,
/// 3 -> 80, 4 -> 64 with some spilling), chosen through the autotuned launch shape. GENERIC = true serves other slabs. CLS: the slabs' shape class - 1 every slab has
/// field_36864's [4, 3] x [2, 3, 8, 64] shapes, 2 field_49152's [4] x [3, 64, 64], 0 any - so that
/// a launch carries only its class's code.
template <bool GENERIC, int CLS, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    crt_batch_kernel(const CrtSlab* __restrict__ slabs, int nslabs, int* counter, int logv, int tile_words) {
    extern __shared__ int64_t smem[];
    __shared__ int s_next;
    for (;;) {
        __syncthreads();  // every thread has read s_next and left the previous slab's tiles
        if (threadIdx.x == 0) s_next = atomicAdd(counter, 1);
        __syncthreads();
        const int si = s_next;
        if (si >= nslabs) return;
        const CrtSlab S = slabs[si];
        const DevPlanHeader* P2 = reinterpret_cast<const DevPlanHeader*>(S.plan2);
        const DevPlanHeader* P3 = reinterpret_cast<const DevPlanHeader*>(S.plan3);
        int64_t* tw2 = smem + tile_words;
        int64_t* tw3 = tw2 + 2 * P2->ntw;
        stage_twiddles(P2, tw2);
        stage_twiddles(P3, tw3);
        __syncthreads();
        if (S.ops & HC_CRT_FORWARD) {
            slab_pass<GENERIC, CLS>(S, P2, tw2, smem, 2, 2, S.kl, logv);
            slab_pass<GENERIC, CLS>(S, P3, tw3, smem, 3, 2, S.kk, logv);
            slab_pass<GENERIC, CLS>(S, P2, tw2, smem, 2, 1, nullptr, logv);
            slab_pass<GENERIC, CLS>(S, P3, tw3, smem, 3, (S.ops & HC_CRT_MUL) ? 3 : 1, nullptr, logv);
        } else if (S.ops & HC_CRT_MUL) {
            const int total = S.dl * S.dk;
            for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
                const int k = idx / S.dk, l = idx - k * S.dk;
                int64_t* x = S.data + k * S.s2 + l;
                *x = mul_mont(*x, S.op[k * S.op_s2 + l], S.n, S.ninv);
            }
            __syncthreads();
        }
        if (S.ops & HC_CRT_INVERSE) {
            slab_pass<GENERIC, CLS>(S, P2, tw2, smem, 2, 2, S.ikl, logv);
            slab_pass<GENERIC, CLS>(S, P3, tw3, smem, 3, 2, S.ikk, logv);
            slab_pass<GENERIC, CLS>(S, P2, tw2, smem, 2, 1, nullptr, logv);
            slab_pass<GENERIC, CLS>(S, P3, tw3, smem, 3, 1, nullptr, logv);
        }
    }
}

}  // namespace

// ---------------------------------------------------------------- plan construction
namespace hc {

/// Builds the stage programs and twiddle tables of CpuNTTPlan::new (src/hal/ntt.rs:561-566,
/// LazyFactorNTT::new :216-281) and simulates the bound tracking of `apply` (:581-657) and of
/// the factor transforms (:301-537).
hc_status build_plan(hc_context ctx, const hc_modulus* m, const size_t* shape, size_t k, hc_ntt_plan* out) {
    (void)ctx;  // plans live in device memory of the current device, shared by its contexts
    const int64_t n = m->n;
    if (n <= 1 || n % 2 == 0 || n >= ((int64_t)1 << 62)) return fail(HC_ERR_ARG, "NTT modulus must be odd and < 2^62");
    HostPlan hp;
    std::memset(&hp.h, 0, sizeof(hp.h));
    hp.h.n = n;
    std::vector<size_t> factors;
    size_t len = 1;
    for (size_t i = 0; i < k; i++) {
        len *= shape[i];
        if (shape[i] > 1) factors.push_back(shape[i]);
    }
    if (len > ((size_t)1 << 30)) return fail(HC_ERR_UNSUPPORTED, "NTT length too large");
    hp.h.len = (int32_t)len;
    int64_t z, u;
    h_barrett(1, n, &z, &u);
    hp.h.one_z = z, hp.h.one_u = u;
    int64_t inv_len = h_pow_mod((int64_t)(len % (size_t)n), (uint64_t)(n - 2), n);
    h_barrett(inv_len, n, &z, &u);
    hp.h.invlen_z = z, hp.h.invlen_u = u;

    u128 fbound = 2 * (u128)n, ibound = 2 * (u128)n;
    size_t suffix = 1;
    for (size_t f : factors) suffix *= f;
    for (size_t fi = 0; fi < factors.size(); fi++) {
        const size_t flen = factors[fi];
        suffix /= flen;
        const bool last_factor = fi + 1 == factors.size();
        const bool r2 = is_pow2(flen);
        if (!r2) {
            size_t l = flen;
            while (l > 1) {
                if (l % 3) return fail(HC_ERR_ARG, "NTT length must be a power of 2 or a power of 3");
                l /= 3;
            }
        }
        if ((n - 1) % (int64_t)flen) return fail(HC_ERR_ARG, "modulus doesn't support roots of unity of this order");
        if (r2 && 2 * (u128)n > I64MAX) return fail(HC_ERR_ARG, "modulus too large for lazy radix-2 butterflies");
        if (!r2 && 3 * (u128)n > I64MAX) return fail(HC_ERR_ARG, "modulus too large for lazy radix-3 butterflies");
        const int radix = r2 ? 2 : 3;
        int64_t root = h_find_root(n, flen);
        int64_t inv_root = h_pow_mod(root, flen - 1, n);
        // twiddles per stage, in the residue-tree order of src/hal/ntt.rs:226-232 / :250-270
        std::vector<std::vector<int64_t>> fw, iv;
        std::vector<size_t> exps{0};
        int64_t zeta = 0, zeta2 = 0;
        if (!r2) {
            zeta = h_pow_mod(root, flen / 3, n);
            zeta2 = h_mul_mod(zeta, zeta, n);
        }
        while (exps.size() < flen) {
            std::vector<int64_t> f1, i1;
            for (size_t e : exps) {
                if (r2) {
                    f1.push_back(h_pow_mod(root, e / 2, n));
                    i1.push_back(h_pow_mod(inv_root, e / 2, n));
                } else {
                    int64_t v = h_pow_mod(root, e / 3, n), v2 = h_mul_mod(v, v, n);
                    f1.push_back(v);
                    f1.push_back(h_mul_mod(zeta, v, n));
                    f1.push_back(h_mul_mod(zeta2, v, n));
                    f1.push_back(v2);
                    f1.push_back(h_mul_mod(zeta, v2, n));
                    f1.push_back(h_mul_mod(zeta2, v2, n));
                    int64_t vi = h_pow_mod(inv_root, e / 3, n);
                    i1.push_back(vi);
                    i1.push_back(h_mul_mod(vi, vi, n));
                }
            }
            fw.push_back(f1);
            iv.push_back(i1);
            std::vector<size_t> next;
            for (size_t e : exps)
                for (int c = 0; c < radix; c++) next.push_back(e / radix + c * (flen / radix));
            exps.swap(next);
        }
        const size_t nst = fw.size();
        int32_t zeta_off = 0;
        if (!r2) {
            zeta_off = hp.next_tw();
            hp.push(zeta);
            hp.push(zeta2);
        }
        // forward program (src/hal/ntt.rs:312-353, :355-411)
        const int fstart = hp.h.nfwd, istart = hp.h.ninv;
        size_t stage_len = flen;
        for (size_t s = 0; s < nst; s++) {
            if (hp.h.nfwd >= HC_MAX_STAGES) return fail(HC_ERR_UNSUPPORTED, "too many NTT stages");
            DevStage& st = hp.h.fwd[hp.h.nfwd++];
            st.radix = radix;
            st.stride = (int32_t)suffix;
            st.flen = (int32_t)flen;
            st.stage_len = (int32_t)stage_len;
            st.tw_off = hp.next_tw();
            for (int64_t v : fw[s]) hp.push(v);
            st.last = last_factor && s + 1 == nst;
            st.span = (int32_t)((stage_len / radix) * suffix);
            st.div_span = make_fastdiv((uint32_t)st.span);
            st.div_nblocks = make_fastdiv((uint32_t)(flen / stage_len));
            const u128 grow = r2 ? (u128)n : 2 * (u128)n;
            if (fbound + grow > I64MAX) {
                st.reduce_before = 1;
                fbound = (u128)n;
            }
            st.skip_ok = (u128)radix * fbound <= I64MAX;
            // the unreduced bound is tracked; a fused final reduction only affects the returned
            // bound of the very last stage, which nothing reads
            fbound = st.skip_ok ? (u128)radix * fbound : fbound + grow;
            stage_len /= radix;
        }
        // inverse program (src/hal/ntt.rs:438-478, :480-533): stages in reverse order
        for (size_t si = nst; si-- > 0;) {
            if (hp.h.ninv >= HC_MAX_STAGES) return fail(HC_ERR_UNSUPPORTED, "too many NTT stages");
            DevStage& st = hp.h.inv[hp.h.ninv++];
            st.radix = radix;
            st.stride = (int32_t)suffix;
            st.flen = (int32_t)flen;
            size_t sl = flen;
            for (size_t q = 0; q < si; q++) sl /= radix;
            st.stage_len = (int32_t)sl;
            st.tw_off = hp.next_tw();
            for (int64_t v : iv[si]) hp.push(v);
            st.zeta_off = zeta_off;
            st.last = last_factor && si == 0;
            st.span = (int32_t)((sl / radix) * suffix);
            st.div_span = make_fastdiv((uint32_t)st.span);
            st.div_nblocks = make_fastdiv((uint32_t)(flen / sl));
            if ((u128)radix * ibound > I64MAX) {
                st.reduce_before = 1;
                ibound = (u128)n;
            }
            ibound = st.last ? (u128)n : (u128)radix * ibound;
        }
        // passes: radix-2 stages in register groups of up to three, radix-3 stages one by one
        auto add_pass = [&](bool fwd, int kind, int k, int first, int span, int glen, int nb) {
            int32_t& cnt = fwd ? hp.h.nfpass : hp.h.nipass;
            DevPass& ps = (fwd ? hp.h.fpass : hp.h.ipass)[cnt++];
            ps.kind = kind, ps.k = k, ps.first = first, ps.span = span, ps.glen = glen, ps.nb = nb;
            ps.div_span = make_fastdiv((uint32_t)(span > 0 ? span : 1));
            ps.div_nb = make_fastdiv((uint32_t)(nb > 0 ? nb : 1));
        };
        const int S = (int)suffix, F = (int)flen, NST = (int)nst;
        for (int c = 0; c < NST;) {
            if (!r2) {
                add_pass(true, 0, 1, fstart + c, 0, 0, 0);
                c++;
                continue;
            }
            int k = std::min(3, NST - c);
            int L = F >> c;  // stage length at the pass's first stage
            add_pass(true, 1, k, fstart + c, (L >> k) * S, L * S, F / L);
            c += k;
        }
        for (int c = 0; c < NST;) {
            if (!r2) {
                add_pass(false, 0, 1, istart + c, 0, 0, 0);
                c++;
                continue;
            }
            int k = std::min(3, NST - c);
            int Lp = 2 << c;  // stage length of the first processed stage (si = nst - 1 - c)
            int Llast = Lp << (k - 1);
            add_pass(false, 1, k, istart + c, (Lp / 2) * S, Llast * S, F / Llast);
            c += k;
        }
    }
    hp.h.ntw = hp.next_tw();
    size_t bytes = sizeof(DevPlanHeader) + hp.tw.size() * sizeof(int64_t);
    std::vector<char> blob(bytes);
    std::memcpy(blob.data(), &hp.h, sizeof(DevPlanHeader));
    if (!hp.tw.empty()) std::memcpy(blob.data() + sizeof(DevPlanHeader), hp.tw.data(), hp.tw.size() * sizeof(int64_t));
    void* dev = nullptr;
    count_alloc();
    if (cudaMalloc(&dev, bytes) != cudaSuccess) return fail(HC_ERR_OOM, "cannot allocate NTT plan");
    hc_status st = cuda_check(cudaMemcpy(dev, blob.data(), bytes, cudaMemcpyHostToDevice), "plan upload");
    if (st != HC_OK) {
        cudaFree(dev);
        return st;
    }
    auto* plan = new hc_ntt_plan_s();
    plan->shape = HC_SHAPE_GENERIC;
    if (factors == std::vector<size_t>{2, 3, 8, 64}) plan->shape = HC_SHAPE_L3072;
    else if (factors == std::vector<size_t>{3, 64, 64}) plan->shape = HC_SHAPE_L12288;
    else if (factors == std::vector<size_t>{4, 3}) plan->shape = HC_SHAPE_C12;
    else if (factors == std::vector<size_t>{4}) plan->shape = HC_SHAPE_C4;
    {
        SchedMasks m{0u, 0u, 0u, 0u, 0u};
        for (int i = 0; i < hp.h.nfwd; i++) {
            m.fred |= (uint32_t)(hp.h.fwd[i].reduce_before != 0) << i;
            m.fskip |= (uint32_t)(hp.h.fwd[i].skip_ok != 0) << i;
            m.flast |= (uint32_t)(hp.h.fwd[i].last != 0) << i;
        }
        for (int i = 0; i < hp.h.ninv; i++) {
            m.ired |= (uint32_t)(hp.h.inv[i].reduce_before != 0) << i;
            m.ilast |= (uint32_t)(hp.h.inv[i].last != 0) << i;
        }
        const SchedMasks f = fixed_masks(plan->shape);
        plan->fixed = plan->shape != HC_SHAPE_GENERIC && m.fred == f.fred && m.fskip == f.fskip &&
                      m.flast == f.flast && m.ired == f.ired && m.ilast == f.ilast;
    }
    plan->dev = dev;
    plan->n = n;
    plan->len = (int32_t)len;
    plan->ntw = hp.h.ntw;
    plan->bytes = bytes;
    *out = plan;
    return HC_OK;
}

hc_status destroy_plan(hc_ntt_plan p) {
    if (!p) return HC_OK;
    cudaFree(p->dev);
    delete p;
    return HC_OK;
}

int64_t plan_modulus(hc_ntt_plan p) { return p->n; }
int32_t plan_len(hc_ntt_plan p) { return p->len; }
const void* plan_device(hc_ntt_plan p) { return p->dev; }
int32_t plan_ntw(hc_ntt_plan p) { return p->ntw; }
int32_t plan_shape(hc_ntt_plan p) { return p->shape | (p->fixed ? 0x100 : 0); }
/// Shared-memory words a slab of the batched transform needs: a padded 3072-residue line, one padded
/// 4096-residue block of a 12288-residue line (line12288_seq), or the generic tile (the whole line,
/// or deg_L' x 2^logv dimension-2 columns); the specialised column passes use none.
size_t crt_slab_tile_words(int32_t shapes, int32_t dl, int32_t dk, int logv) {
    const int s3 = shapes & 0xff, s2 = (shapes >> 8) & 0xff;
    const bool f3 = (shapes >> 16) & 1, f2 = (shapes >> 17) & 1;
    const size_t w3 = !f3 ? (size_t)dk
                          : s3 == HC_SHAPE_L3072 ? (size_t)line_tile_words(HC_SHAPE_L3072)
                          : s3 == HC_SHAPE_L12288 ? (size_t)(4096 + 4096 / 8) : (size_t)dk;
    const size_t w2 = f2 && (s2 == HC_SHAPE_C12 || s2 == HC_SHAPE_C4) ? 0 : ((size_t)dl << logv);
    const size_t w = std::max(w3, w2);
    return (w + 1) & ~(size_t)1;
}

int32_t plan_tile_words(hc_ntt_plan p) {
    return p->shape == HC_SHAPE_L3072 || p->shape == HC_SHAPE_L12288 ? line_tile_words(p->shape) : 0;
}

/// Launches the persistent batched-transform kernel over `nslabs` device slab descriptors.
/// `tile_words`: largest tile (deg_K, or deg_L' x 2^logv); `tw_words`: largest pair of twiddle
/// tables (dimension-2 + dimension-3 plan) of a slab. `counter` is reset on the stream first.
/// Whether a slab runs entirely on the specialised line and column code (crt_batch_kernel<false>).
bool crt_slab_specialised(int32_t shapes) {
    const int s3 = shapes & 0xff, s2 = (shapes >> 8) & 0xff;
    return ((shapes >> 16) & 1) && (s3 == HC_SHAPE_L3072 || s3 == HC_SHAPE_L12288) && ((shapes >> 17) & 1) &&
           (s2 == HC_SHAPE_C12 || s2 == HC_SHAPE_C4);
}

/// The specialised kernel of class CLS for a launch shape.
template <int CLS>
auto crt_batch_variant(const CrtLaunch& L) {
    return L.ctas_per_sm >= 4   ? crt_batch_kernel<false, CLS, 256, 4>
           : L.ctas_per_sm == 3 ? crt_batch_kernel<false, CLS, 256, 3>
                                : crt_batch_kernel<false, CLS, 256, 2>;
}

/// Shape class of specialised slab shapes (crt_batch_kernel's CLS): 1 field_36864, 2 field_49152
/// (CLS 0: a launch over both).
int crt_slab_kernel_class(int32_t shapes) { return (shapes & 0xff) == HC_SHAPE_L3072 ? 1 : 2; }

hc_status launch_crt_batch(hc_context ctx, const CrtSlab* slabs, int nslabs, int* counter, size_t tile_words,
                           size_t tw_words, const CrtLaunch& L, bool generic, int cls) {
    if (nslabs <= 0) return HC_OK;
    auto kern = generic    ? crt_batch_kernel<true, 0, 256, 2>
                : cls == 1 ? crt_batch_variant<1>(L)
                : cls == 2 ? crt_batch_variant<2>(L)
                           : crt_batch_variant<0>(L);
    if (L.threads < 32 || L.threads > 256 || L.threads % 32) return fail(HC_ERR_ARG, "batched transform: threads per CTA");
    if (L.logv < 0 || L.logv > 6) return fail(HC_ERR_ARG, "batched transform: dimension-2 tile width");
    const size_t smem = (tile_words + tw_words) * 8;
    if (smem > max_smem_optin(ctx)) return fail(HC_ERR_UNSUPPORTED, "batched transform: slab tiles exceed shared memory");
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_check(e, "batched transform smem attribute");
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, L.threads, smem);
    if (e != cudaSuccess) return cuda_check(e, "batched transform occupancy");
    if (occ < 1) return fail(HC_ERR_UNSUPPORTED, "batched transform: launch shape does not fit an SM");
    int per = L.ctas_per_sm < 1 ? 1 : (L.ctas_per_sm < occ ? L.ctas_per_sm : occ);
    int64_t grid = (int64_t)num_sms(ctx) * per;
    if (grid > nslabs) grid = nslabs;
    hc_status st = cuda_check(cudaMemsetAsync(counter, 0, sizeof(int), stream_of(ctx)), "batched transform counter");
    if (st) return st;
    kern<<<(unsigned)grid, (unsigned)L.threads, smem, stream_of(ctx)>>>(slabs, nslabs, counter, L.logv,
                                                                      (int)tile_words);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "batched transform launch");
}

/// Launches the tile kernel for one HAL NTT call (mode 0 ntt, 1 intt, 2 ntt_mul).
/// Whether launch_ntt runs a call on the specialised column kernel, the one form that can read a
/// separate source (launch_ntt's `src`).
bool ntt_column_path(const hc_ntt_plan* plans, size_t nplans, int dim) {
    if (dim != 2 || nplans == 0 || !plans[0]) return false;
    const int shape = plans[0]->shape;
    int32_t max_tw = 0;
    for (size_t j = 0; j < nplans; j++) {
        if (!plans[j] || plans[j]->shape != shape) return false;
        max_tw = std::max(max_tw, plans[j]->ntw);
    }
    return (shape == HC_SHAPE_C12 || shape == HC_SHAPE_C4) && 2 * max_tw <= HC_COL_TW;
}

hc_status launch_ntt(hc_context ctx, const KView& t, const hc_ntt_plan* plans, size_t nplans, int dim, int mode,
                     const KView& mul, const KMods& mods, const KView* src) {
    if (src && !ntt_column_path(plans, nplans, dim)) return fail(HC_ERR_UNSUPPORTED, "out-of-place NTT form");
    if ((int64_t)nplans != t.n1) return fail(HC_ERR_SHAPE, "one NTT plan per RNS row required");
    if (nplans > HC_MAX_MODS) return fail(HC_ERR_UNSUPPORTED, "too many RNS rows in one call");
    const int64_t len = dim == 3 ? t.n3 : t.n2;
    PlanPtrs pp;
    int32_t max_tw = 0;
    for (size_t j = 0; j < nplans; j++) {
        if (!plans[j]) return fail(HC_ERR_ARG, "null NTT plan");
        if (plans[j]->len != len) return fail(HC_ERR_SHAPE, "NTT plan length does not match the transformed dimension");
        pp.p[j] = reinterpret_cast<const DevPlanHeader*>(plans[j]->dev);
        max_tw = std::max(max_tw, plans[j]->ntw);
    }
    if (t.n0 == 0 || t.n1 == 0 || t.n2 == 0 || t.n3 == 0) return HC_OK;
    int shape = plans[0]->shape;
    for (size_t j = 1; j < nplans; j++)
        if (plans[j]->shape != shape) shape = HC_SHAPE_GENERIC;
    bool fix = true;
    for (size_t j = 0; j < nplans; j++) fix = fix && plans[j]->fixed;
    if (dim == 3 && (shape == HC_SHAPE_L3072 || shape == HC_SHAPE_L12288)) {
        const size_t smem = ((size_t)line_tile_words(shape) + (shape == HC_SHAPE_L3072 ? 0 : 2 * (size_t)max_tw)) * 8;
        const int64_t tiles = t.n0 * t.n1 * t.n2;
        if (smem <= max_smem_optin(ctx) && tiles <= 0x7fffffff) {
            if (shape == HC_SHAPE_L3072)
                return launch_special_mode<HC_SHAPE_L3072>(ctx, mode, fix, t, pp, mul, mods, smem, tiles, 0);
            return launch_special_mode<HC_SHAPE_L12288>(ctx, mode, fix, t, pp, mul, mods, smem, tiles, 0);
        }
    }
    if (dim == 2 && (shape == HC_SHAPE_C12 || shape == HC_SHAPE_C4) && 2 * max_tw <= HC_COL_TW) {
        const int64_t ncb = (t.n3 + HC_COL_THREADS - 1) / HC_COL_THREADS;
        const int64_t tiles = t.n0 * t.n1 * ncb;
        if (tiles <= 0x7fffffff) {
            if (shape == HC_SHAPE_C12)
                return launch_special_mode<HC_SHAPE_C12>(ctx, mode, fix, t, pp, mul, mods, 0, tiles, (int)ncb,
                                                         src ? *src : KView());
            return launch_special_mode<HC_SHAPE_C4>(ctx, mode, fix, t, pp, mul, mods, 0, tiles, (int)ncb,
                                                    src ? *src : KView());
        }
    }
    if (src) return fail(HC_ERR_UNSUPPORTED, "out-of-place NTT form");
    int V = 1, logv = 0;
    int64_t ntile2 = 1;
    if (dim == 2) {
        // as many dimension-3 columns per tile as fit into 48 KB of shared memory (<= 64)
        V = 64;
        while (V > 1 && (len * V * 8 > 49152 || V / 2 >= t.n3)) V /= 2;
        while ((1 << logv) < V) logv++;
        ntile2 = (t.n3 + V - 1) / V;
    }
    const size_t tw_bytes = (size_t)max_tw * 16;
    size_t smem = (size_t)len * V * 8 + tw_bytes;
    int use_smem = 1;
    size_t maxs = max_smem_optin(ctx);
    if (smem > maxs) {
        if (dim == 2) return fail(HC_ERR_UNSUPPORTED, "dimension-2 NTT length too large");
        use_smem = 0;
        smem = tw_bytes;
        if (smem > maxs) return fail(HC_ERR_UNSUPPORTED, "NTT twiddle table too large");
    }
    if (smem > 49152) {
        cudaError_t e = cudaFuncSetAttribute(ntt_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_check(e, "ntt smem attribute");
    }
    int64_t tiles = dim == 3 ? t.n0 * t.n1 * t.n2 : t.n0 * t.n1 * ntile2;
    if (tiles > 0x7fffffff) return fail(HC_ERR_UNSUPPORTED, "too many NTT tiles in one call");
    // about 24 elements (three groups of eight) per thread, 64..256 threads
    int64_t threads = ((len * V / 24) + 31) / 32 * 32;
    threads = threads < 64 ? 64 : (threads > 256 ? 256 : threads);
    ntt_tile_kernel<<<(unsigned)tiles, (unsigned)threads, smem, stream_of(ctx)>>>(t, pp, dim, mode, mul, mods, logv,
                                                                    (int)ntile2, use_smem);
    count_launch(ctx);
    return cuda_check(cudaGetLastError(), "ntt kernel launch");
}

}  // namespace hc
