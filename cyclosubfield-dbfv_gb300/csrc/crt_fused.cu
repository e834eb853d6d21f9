// Fused CRT-transform passes of field_49152: both dimensions' NTTs of one half of pb_to_crt /
// crt_to_pb in one launch.
//
// The reference transforms a batch [count, r, deg_L', deg_K] in four HAL calls
// (src/ring.rs:1118-1161): ntt_mul along dimension 2 (deg_L' columns, times the kernel K_L'),
// ntt_mul along dimension 3 (deg_K lines, times K_K), intt along dimension 2, intt along
// dimension 3. Each call reads and writes the whole batch. Here each (element, factor) slab of
// field_49152 - 4 rows ([4]) of 12288 residues ([3, 64, 64]), 393 KB, more than one SM's shared
// memory - is held by a cluster of 12 CTAs in distributed shared memory, CTA 3k + b owning block b
// (4096 residues) of row k, and one launch runs a dimension-2 pass and the following dimension-3
// pass of every slab:
//   launch A: ntt_mul along dimension 2, then ntt_mul along dimension 3;
//   launch B: intt along dimension 2, then intt along dimension 3 (times an optional factor, the
//             caller's next Montgomery product).
// Phase 1: the cluster's threads read positions p, p + 4096, p + 8192 of all four rows (12
// residues; coalesced along dimension 3), run the four-point column transforms and then the
// leading radix-3 stage of each row, which couples exactly those three positions, and store each
// result into the shared memory of the CTA owning its (row, block). A cluster barrier makes the
// stores visible. Phase 2: every CTA runs the remaining twelve radix-2 stages of its block in its
// own shared memory and stores it. The slab is read once and written once per launch, so a
// transform moves half the bytes of the four-call form and launches half the kernels.
// Butterflies, their order and the reduction / skip / fused-final schedule are exactly those of
// the single-dimension kernels (ntt_fast.cuh), so the results are bit-identical.
#include <cooperative_groups.h>

#include <map>
#include <mutex>

#include "common.cuh"
#include "ntt_plan.cuh"

namespace cg = cooperative_groups;

namespace hc {
const void* plan_device(hc_ntt_plan p);
int32_t plan_shape(hc_ntt_plan p);
}  // namespace hc

namespace {

constexpr int CLUSTER = 12;  // CTAs per slab
constexpr int THREADS = 128;
constexpr size_t SMEM12288 = 4608 * 8;  // one padded 4096-residue block

/// Split cluster barrier: every CTA arrives when it starts and waits before its first store into
/// another CTA's shared memory, which is then known to be running (the loads and arithmetic of
/// the first positions overlap the wait).
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait;\n" ::: "memory"); }



/// The four-point factor of a dimension-2 column ([4] or the [4] of [4, 3]: its two radix-2
/// stages f0, f1) for the two output rows {2h, 2h + 1} only, from the four inputs x0..x3: the
/// same integers as ntt_fast.cuh's col12 / col4 (and the reference's butterflies,
/// src/hal/ntt.rs:338-349, :465-476). Two warps share a column, one per h, so that each keeps
/// six of the twelve values of a [4, 3] column (or of three [4] columns) in registers; the
/// duplicated work is the four-point factor's one Barrett product per column.
template <bool INV>
__device__ __forceinline__ void four_half(const fast::Ctx& c, const fast::SF& f0, const fast::SF& f1, int h,
                                          int64_t x0, int64_t x1, int64_t x2, int64_t x3, int64_t& o0, int64_t& o1) {
    if (f0.red) {
        x0 = fast::red1(c, x0), x1 = fast::red1(c, x1), x2 = fast::red1(c, x2), x3 = fast::red1(c, x3);
    }
    if (!INV) {
        // stage 0 (length 4, block 0): pairs (0, 2), (1, 3)
        int64_t t02 = x2, t13 = x3;
        if (!f0.skip_ok) {
            int64_t z, u;
            fast::twl(c, f0.tw_off, z, u);
            t02 = bmul(z, u, x2, c.n), t13 = bmul(z, u, x3, c.n);
        }
        int64_t p = h ? wsub(x0, t02) : wadd(x0, t02), q = h ? wsub(x1, t13) : wadd(x1, t13);
        if (f1.red) p = fast::red1(c, p), q = fast::red1(c, q);
        // stage 1 (length 2): block 0 = rows (0, 1), block 1 = rows (2, 3)
        int64_t t = q;
        if (h) {
            int64_t z, u;
            fast::twl(c, f1.tw_off + 1, z, u);
            t = bmul(z, u, q, c.n);
        } else if (!f1.skip_ok) {
            int64_t z, u;
            fast::twl(c, f1.tw_off, z, u);
            t = bmul(z, u, q, c.n);
        }
        o0 = wadd(p, t), o1 = wsub(p, t);
    } else {
        // stage 0 (length 2): block 0 = (0, 1), block 1 = (2, 3)
        int64_t y0 = wadd(x0, x1), y1 = wsub(x0, x1), y2 = wadd(x2, x3), y3 = wsub(x2, x3);
        if (f0.last) {
            y0 = bmul(c.il_z, c.il_u, y0, c.n), y1 = bmul(c.il_z, c.il_u, y1, c.n);
            y2 = bmul(c.il_z, c.il_u, y2, c.n), y3 = bmul(c.il_z, c.il_u, y3, c.n);
        } else {
            int64_t z, u;
            fast::twl(c, f0.tw_off + 1, z, u);
            if (z != 1) y3 = bmul(z, u, y3, c.n);
        }
        if (f1.red) {
            y0 = fast::red1(c, y0), y1 = fast::red1(c, y1), y2 = fast::red1(c, y2), y3 = fast::red1(c, y3);
        }
        // stage 1 (length 4): pairs (0, 2), (1, 3)
        o0 = h ? wsub(y0, y2) : wadd(y0, y2), o1 = h ? wsub(y1, y3) : wadd(y1, y3);
        if (f1.last) o0 = bmul(c.il_z, c.il_u, o0, c.n), o1 = bmul(c.il_z, c.il_u, o1, c.n);
    }
}

/// Fused pass of a field_49152 slab: CTA 3k + b of the cluster owns block b of row k.
template <int DIR, bool POST>
__global__ void __launch_bounds__(THREADS, 6)
    crt_slab12288_kernel(KView t, KView src, PlanPtrs p2, PlanPtrs p3, KView m2, KView m3, KMods mods, int reverse) {
    extern __shared__ int64_t smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int row = rank / 3, blk = rank - 3 * (rank / 3);
    // reverse: the last slab first, so that the clusters scheduled first read what the producer
    // of the input (or the other half of the transform) wrote last, still in L2
    const int64_t slab = reverse ? gridDim.x / CLUSTER - 1 - blockIdx.x / CLUSTER : blockIdx.x / CLUSTER;
    const int64_t j = slab % t.n1, i = slab / t.n1;
    const DevPlanHeader* P2 = p2.p[j];
    const DevPlanHeader* P3 = p3.p[j];
    const int64_t n = mods.n[j], ninv = mods.ninv[j];
    constexpr bool inv = DIR == 1;
    const fast::Ctx c3 = make_ctx(P3, reinterpret_cast<const int64_t*>(P3 + 1));
    const FixedSched<HC_SHAPE_L12288, inv> sch3{inv ? P3->inv : P3->fwd};
    cluster_arrive_relaxed();
    // ---- phase 1: positions p, p + 4096, p + 8192 of the four rows, over the cluster's threads;
    // warp w keeps rows 2h, 2h + 1 (h = w & 1) of 64 positions per CTA and step
    {
        const fast::Ctx c2 = make_ctx(P2, reinterpret_cast<const int64_t*>(P2 + 1));
        const FixedSched<HC_SHAPE_C4, inv> sch2{inv ? P2->inv : P2->fwd};
        const fast::SF f0 = fast::sflags(sch2, 0), f1 = fast::sflags(sch2, 1);
        const fast::SF f30 = fast::sflags(sch3, 0);
        const int warp = threadIdx.x >> 5, h = warp & 1;
        int64_t m2a = 0, m2b = 0;  // the dimension-2 multipliers of rows 2h, 2h + 1
        if (DIR == 0) m2a = *kat<int64_t>(m2, i, j, 2 * h, 0), m2b = *kat<int64_t>(m2, i, j, 2 * h + 1, 0);
        const int64_t* gs = reinterpret_cast<const int64_t*>(src.p) + i * src.s0 + j * src.s1;
#pragma unroll 1
        for (int q = 0;; q++) {
            const int p = 768 * q + 64 * rank + 32 * (warp >> 1) + (threadIdx.x & 31);
            if (p >= 4096) break;  // warp-uniform (4096 and 768 are multiples of 32)
            int64_t y[2][3];  // rows 2h, 2h + 1 by block b
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const int64_t* col = gs + 4096 * b + p;
                four_half<inv>(c2, f0, f1, h, col[0], col[src.s2], col[2 * src.s2], col[3 * src.s2], y[0][b], y[1][b]);
                if (DIR == 0) y[0][b] = mul_mont(y[0][b], m2a, n, ninv), y[1][b] = mul_mont(y[1][b], m2b, n, ninv);
            }
#pragma unroll
            for (int a = 0; a < 2; a++) {
                if (f30.red) {
#pragma unroll
                    for (int b = 0; b < 3; b++) y[a][b] = fast::red1(c3, y[a][b]);
                }
                if (inv) fast::inv3(c3, f30, y[a][0], y[a][1], y[a][2]);
                else fast::fwd3<true>(c3, f30, false, 0, y[a][0], y[a][1], y[a][2]);
            }
            if (q == 0) cluster_wait();  // every thread runs q = 0 (p < 768)
#pragma unroll
            for (int a = 0; a < 2; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) cluster.map_shared_rank(smem, 3 * (2 * h + a) + b)[fast::pad8(p)] = y[a][b];
        }
    }
    cluster.sync();
    // ---- phase 2: stages 1..12 of block `blk` of row `row`, in this CTA's shared memory
    if (!inv) {
        fast::r2_pass<false, 3, 9, 12, 0>(c3, smem, 512, sch3, 1, false);  // factor 64 (a): 2048, 1024, 512
        __syncthreads();
        fast::r2_pass<false, 3, 6, 9, 3>(c3, smem, 512, sch3, 4, false);   // factor 64 (a): 256, 128, 64
        __syncthreads();
        fast::r2_pass<false, 3, 3, 6, 0>(c3, smem, 512, sch3, 7, false);   // factor 64 (b): 32, 16, 8
        __syncthreads();
        fast::r2_pass<false, 3, 0, 3, 3>(c3, smem, 512, sch3, 10, false);  // factor 64 (b): 4, 2, 1
    } else {
        fast::r2_pass<true, 3, 6, 9, 3>(c3, smem, 512, sch3, 1, false);    // factor 64 (a): 64, 128, 256
        __syncthreads();
        fast::r2_pass<true, 3, 9, 12, 0>(c3, smem, 512, sch3, 4, false);   // factor 64 (a): 512, 1024, 2048
        __syncthreads();
        fast::r2_pass<true, 3, 0, 3, 3>(c3, smem, 512, sch3, 7, false);    // factor 64 (b): 1, 2, 4
        __syncthreads();
        fast::r2_pass<true, 3, 3, 6, 0>(c3, smem, 512, sch3, 10, false);   // factor 64 (b): 8, 16, 32
    }
    __syncthreads();
    int64_t* g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + row * t.s2 + 4096 * blk;
    const int64_t* mulp = nullptr;
    int64_t me = 0;
    if (DIR == 0 || POST) {
        me = m3.b3 ? 0 : 1;
        mulp = kat<int64_t>(m3, i, j, row, 0) + (me ? 4096 * blk : 0);
    }
    fast::line_store(smem, g, 4096, DIR == 0 || POST, mulp, me, n, ninv);
}

template <class K>
hc_status cluster_launch(hc_context ctx, K kern, int64_t slabs, size_t smem, const KView& t, const KView& src,
                         const PlanPtrs& p2, const PlanPtrs& p3, const KView& m2, const KView& m3, const KMods& mods,
                         int reverse) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(slabs * CLUSTER), 1, 1);
    cfg.blockDim = dim3(THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = hc::stream_of(ctx);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    hc_status st = hc::cuda_check(cudaLaunchKernelEx(&cfg, kern, t, src, p2, p3, m2, m3, mods, reverse), "fused CRT pass launch");
    hc::count_launch(ctx);
    return st;
}

/// Sets the kernel's attributes (shared memory, a 12-CTA cluster) and tells whether at least one
/// such cluster fits the device; done once per kernel and device.
template <class K>
bool cluster_ready(K kern, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, bool> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair((const void*)kern, dev);
    auto it = done.find(key);
    if (it != done.end()) return it->second;
    bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess &&
              cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    if (ok) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CLUSTER, 1, 1);
        cfg.blockDim = dim3(THREADS, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CLUSTER;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        ok = cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) == cudaSuccess && clusters > 0;
    }
    cudaGetLastError();  // a refused attribute leaves no sticky error behind
    done[key] = ok;
    return ok;
}

template <int DIR, bool POST>
hc_status launch_fused(hc_context ctx, int64_t slabs, const KView& t, const KView& src, const PlanPtrs& p2,
                       const PlanPtrs& p3, const KView& m2, const KView& m3, const KMods& mods, int reverse) {
    return cluster_launch(ctx, crt_slab12288_kernel<DIR, POST>, slabs, SMEM12288, t, src, p2, p3, m2, m3, mods, reverse);
}

/// Whether a transform's plans are field_49152's shapes ([4] along dimension 2, [3, 64, 64] along
/// dimension 3) with their compiled-in schedules and t has their extents. (field_36864's [4, 3] x
/// [2, 3, 8, 64] slabs run faster as separate column and line launches: there the column pass
/// is a cheap HBM-bound kernel, and the fused form measured 0.92 ms per transform of a
/// [24, 34, 12, 3072] tensor against 0.88 ms for the four launches.)
bool fused_shape(const hc_ntt_plan* plans2, const hc_ntt_plan* plans3, size_t r, const KView& t) {
    if (r == 0 || r > HC_MAX_MODS || (int64_t)r != t.n1) return false;
    const int s2 = hc::plan_shape(plans2[0]), s3 = hc::plan_shape(plans3[0]);
    if (s2 != (HC_SHAPE_C4 | 0x100) || s3 != (HC_SHAPE_L12288 | 0x100) || t.n2 != 4 || t.n3 != 12288) return false;
    for (size_t j = 1; j < r; j++)
        if (hc::plan_shape(plans2[j]) != s2 || hc::plan_shape(plans3[j]) != s3) return false;
    return t.n0 * t.n1 * CLUSTER <= 0x7fffffff;
}

}  // namespace

namespace hc {

/// Whether the fused passes can run this transform: the plans are the fused shapes (fused_shape)
/// and the device runs the 12-CTA clusters of all three kernels of that shape.
bool crt_pass_ready(hc_context ctx, const hc_ntt_plan* plans2, const hc_ntt_plan* plans3, size_t r, const KView& t) {
    (void)ctx;
    return fused_shape(plans2, plans3, r, t) && cluster_ready(crt_slab12288_kernel<0, false>, SMEM12288) &&
           cluster_ready(crt_slab12288_kernel<1, false>, SMEM12288) &&
           cluster_ready(crt_slab12288_kernel<1, true>, SMEM12288);
}

/// One fused half of a CRT transform over t [count, r, deg_L', deg_K] (dimension 3 contiguous):
/// dir 0 = ntt_mul along dimension 2 by m2, then along dimension 3 by m3 (reading the input from
/// src when given: the caller's copy folded into phase 1; src must not overlap t other than
/// exactly); dir 1 = intt along dimension 2, then along dimension 3, times m3 when `post`.
/// The caller checks crt_pass_ready first.
hc_status launch_crt_pass(hc_context ctx, int dir, const KView& t, const KView* src, const hc_ntt_plan* plans2,
                          const hc_ntt_plan* plans3, size_t r, const KView& m2, const KView& m3, bool post,
                          const KMods& mods) {
    if (!fused_shape(plans2, plans3, r, t)) return fail(HC_ERR_UNSUPPORTED, "fused CRT pass: plans are not a fused shape");
    PlanPtrs p2, p3;
    for (size_t j = 0; j < r; j++) {
        p2.p[j] = reinterpret_cast<const DevPlanHeader*>(plan_device(plans2[j]));
        p3.p[j] = reinterpret_cast<const DevPlanHeader*>(plan_device(plans3[j]));
    }
    const int64_t slabs = t.n0 * t.n1;
    if (slabs == 0) return HC_OK;
    const KView& s = src ? *src : t;
    // the first half runs the slabs last to first (the input's producer wrote them first to last),
    // the second half first to last (the first half wrote them last to first)
    if (dir == 0) return launch_fused<0, false>(ctx, slabs, t, s, p2, p3, m2, m3, mods, 1);
    if (post) return launch_fused<1, true>(ctx, slabs, t, s, p2, p3, m2, m3, mods, 0);
    return launch_fused<1, false>(ctx, slabs, t, s, p2, p3, m2, m3, mods, 0);
}

}  // namespace hc
