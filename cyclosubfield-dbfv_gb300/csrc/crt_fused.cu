// Fused CRT-transform passes of the two large field descriptors: both dimensions' NTTs of one
// half of pb_to_crt / crt_to_pb in one launch.
//
// The reference transforms a batch [count, r, deg_L', deg_K] in four HAL calls
// (src/ring.rs:1118-1161): ntt_mul along dimension 2 (deg_L' columns, times the kernel K_L'),
// ntt_mul along dimension 3 (deg_K lines, times K_K), intt along dimension 2, intt along
// dimension 3. Each call reads and writes the whole batch. Here each (element, factor) slab -
// deg_L' x deg_K residues, 295 KB (field_36864) or 393 KB (field_49152), more than one SM's shared
// memory - is held by a cluster of 12 CTAs in distributed shared memory, and one launch runs a
// dimension-2 pass and the following dimension-3 pass of every slab:
//   launch A: ntt_mul along dimension 2, then ntt_mul along dimension 3;
//   launch B: intt along dimension 2, then intt along dimension 3 (times an optional factor, the
//             caller's next Montgomery product).
// Phase 1: each CTA reads a range of positions of all deg_L' rows of its slab from global memory
// (coalesced along dimension 3), runs the column transforms in registers and stores every output
// into the shared memory of the CTA that owns that row (or row block). A cluster barrier makes
// the stores visible. Phase 2: every CTA runs the line transform of its row (block) in its own
// shared memory and stores it. The slab is read once and written once per launch, so a transform
// moves half the bytes of the four-call form and launches half the kernels. Butterflies, their
// order and the reduction / skip / fused-final schedule are exactly those of the single-dimension
// kernels (ntt_fast.cuh), so the results are bit-identical.
//
//   field_36864: rows [4, 3] (12), lines [2, 3, 8, 64] (3072). CTA k of the cluster owns row k;
//     phase 1 covers 256 positions per CTA; phase 2 is the line kernel's programme.
//   field_49152: rows [4] (4), lines [3, 64, 64] (12288). CTA 3k + b owns block b (4096 residues)
//     of row k. Phase 1 takes positions p, p + 4096, p + 8192 of all four rows (12 residues), runs
//     the four-point column transforms and then the leading radix-3 stage of each row (which
//     couples exactly those three positions), so phase 2 - the twelve radix-2 stages - stays
//     inside each CTA's block.
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
constexpr size_t SMEM3072 = (size_t)line_tile_words(HC_SHAPE_L3072) * 8;  // one padded line
constexpr size_t SMEM12288 = 4608 * 8;                                    // one padded 4096-residue block

/// Split cluster barrier: every CTA arrives when it starts and waits before its first store into
/// another CTA's shared memory, which is then known to be running (the loads and arithmetic of
/// the first positions overlap the wait).
__device__ __forceinline__ void cluster_arrive_relaxed() { asm volatile("barrier.cluster.arrive.relaxed;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait;\n" ::: "memory"); }

/// Fused pass of a field_36864 slab (DIR 0: launch A, DIR 1: launch B). src: read in phase 1
/// (t itself for an in-place call). m2: the dimension-2 multiplier [1, r, 12, 1] (DIR 0); m3: the
/// dimension-3 multiplier, [1, r, 1, 3072] (DIR 0) or a broadcast factor (DIR 1 with POST).
template <int DIR, bool POST>
__global__ void __launch_bounds__(THREADS, 8)
    crt_slab3072_kernel(KView t, KView src, PlanPtrs p2, PlanPtrs p3, KView m2, KView m3, KMods mods) {
    extern __shared__ int64_t smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();  // the row this CTA owns
    const int64_t slab = blockIdx.x / CLUSTER;
    const int64_t j = slab % t.n1, i = slab / t.n1;
    const DevPlanHeader* P2 = p2.p[j];
    const DevPlanHeader* P3 = p3.p[j];
    const int64_t n = mods.n[j], ninv = mods.ninv[j];
    constexpr bool inv = DIR == 1;
    cluster_arrive_relaxed();
    // ---- phase 1: 12-residue columns at positions [256 rank, 256 rank + 256)
    {
        const fast::Ctx c2 = make_ctx(P2, reinterpret_cast<const int64_t*>(P2 + 1));
        const FixedSched<HC_SHAPE_C12, inv> sch{inv ? P2->inv : P2->fwd};
        fast::SF f[3];
#pragma unroll
        for (int q = 0; q < 3; q++) f[q] = fast::sflags(sch, q);
        const int64_t* gs = reinterpret_cast<const int64_t*>(src.p) + i * src.s0 + j * src.s1;
        bool first = true;
        for (int l = 256 * rank + threadIdx.x; l < 256 * rank + 256; l += THREADS) {
            int64_t x[4][3];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[a][b] = gs[(3 * a + b) * src.s2 + l];
            fast::col12(c2, f, inv, false, x);
            if (first) {  // every thread runs the first iteration (256 positions, 128 threads)
                cluster_wait();
                first = false;
            }
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    int64_t v = x[a][b];
                    if (DIR == 0) v = mul_mont(v, *kat<int64_t>(m2, i, j, 3 * a + b, 0), n, ninv);
                    cluster.map_shared_rank(smem, 3 * a + b)[fast::pad8(l)] = v;
                }
        }
    }
    cluster.sync();  // every row of the slab is in its owner's shared memory
    // ---- phase 2: the line of row `rank`
    {
        const fast::Ctx c3 = make_ctx(P3, reinterpret_cast<const int64_t*>(P3 + 1));
        const FixedSched<HC_SHAPE_L3072, inv> sch{inv ? P3->inv : P3->fwd};
        int64_t* g = reinterpret_cast<int64_t*>(t.p) + i * t.s0 + j * t.s1 + rank * t.s2;
        const int64_t* mulp = nullptr;
        int64_t me = 0;
        if (DIR == 0 || POST) {
            mulp = kat<int64_t>(m3, i, j, rank, 0);
            me = m3.b3 ? 0 : 1;
        }
        if (DIR == 0) fast::line3072<2, decltype(sch), true>(sch, c3, smem, g, mulp, me, n, ninv);
        else if (POST) fast::line3072<3, decltype(sch), true>(sch, c3, smem, g, mulp, me, n, ninv);
        else fast::line3072<1, decltype(sch), true>(sch, c3, smem, g, mulp, me, n, ninv);
    }
}

/// Fused pass of a field_49152 slab: CTA 3k + b of the cluster owns block b of row k.
template <int DIR, bool POST>
__global__ void __launch_bounds__(THREADS, 6)
    crt_slab12288_kernel(KView t, KView src, PlanPtrs p2, PlanPtrs p3, KView m2, KView m3, KMods mods) {
    extern __shared__ int64_t smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int row = rank / 3, blk = rank - 3 * (rank / 3);
    const int64_t slab = blockIdx.x / CLUSTER;
    const int64_t j = slab % t.n1, i = slab / t.n1;
    const DevPlanHeader* P2 = p2.p[j];
    const DevPlanHeader* P3 = p3.p[j];
    const int64_t n = mods.n[j], ninv = mods.ninv[j];
    constexpr bool inv = DIR == 1;
    const fast::Ctx c3 = make_ctx(P3, reinterpret_cast<const int64_t*>(P3 + 1));
    const FixedSched<HC_SHAPE_L12288, inv> sch3{inv ? P3->inv : P3->fwd};
    cluster_arrive_relaxed();
    // ---- phase 1: positions p, p + 4096, p + 8192 of the four rows, over the cluster's threads
    {
        const fast::Ctx c2 = make_ctx(P2, reinterpret_cast<const int64_t*>(P2 + 1));
        const FixedSched<HC_SHAPE_C4, inv> sch2{inv ? P2->inv : P2->fwd};
        fast::SF f2[2];
        f2[0] = fast::sflags(sch2, 0), f2[1] = fast::sflags(sch2, 1);
        const fast::SF f30 = fast::sflags(sch3, 0);
        int64_t m2v[4] = {0, 0, 0, 0};
        if (DIR == 0) {
#pragma unroll
            for (int k = 0; k < 4; k++) m2v[k] = *kat<int64_t>(m2, i, j, k, 0);
        }
        const int64_t* gs = reinterpret_cast<const int64_t*>(src.p) + i * src.s0 + j * src.s1;
        bool first = true;
        for (int p = rank * THREADS + threadIdx.x; p < 4096; p += CLUSTER * THREADS) {
            int64_t x[4][3];  // [row][block]
#pragma unroll
            for (int k = 0; k < 4; k++)
#pragma unroll
                for (int b = 0; b < 3; b++) x[k][b] = gs[k * src.s2 + 4096 * b + p];
#pragma unroll
            for (int b = 0; b < 3; b++) {
                int64_t col[4] = {x[0][b], x[1][b], x[2][b], x[3][b]};
                fast::col4(c2, f2, inv, false, col);
#pragma unroll
                for (int k = 0; k < 4; k++) x[k][b] = DIR == 0 ? mul_mont(col[k], m2v[k], n, ninv) : col[k];
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (f30.red) {
#pragma unroll
                    for (int b = 0; b < 3; b++) x[k][b] = fast::red1(c3, x[k][b]);
                }
                if (inv) fast::inv3(c3, f30, 0, x[k][0], x[k][1], x[k][2]);
                else fast::fwd3<true>(c3, f30, false, 0, x[k][0], x[k][1], x[k][2]);
            }
            if (first) {  // every thread runs the first iteration (4096 positions, 1536 threads)
                cluster_wait();
                first = false;
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
#pragma unroll
                for (int b = 0; b < 3; b++) cluster.map_shared_rank(smem, 3 * k + b)[fast::pad8(p)] = x[k][b];
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
                         const PlanPtrs& p2, const PlanPtrs& p3, const KView& m2, const KView& m3, const KMods& mods) {
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
    hc_status st = hc::cuda_check(cudaLaunchKernelEx(&cfg, kern, t, src, p2, p3, m2, m3, mods), "fused CRT pass launch");
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
hc_status launch_shape(hc_context ctx, int shape3, int64_t slabs, const KView& t, const KView& src,
                       const PlanPtrs& p2, const PlanPtrs& p3, const KView& m2, const KView& m3, const KMods& mods) {
    if (shape3 == HC_SHAPE_L3072)
        return cluster_launch(ctx, crt_slab3072_kernel<DIR, POST>, slabs, SMEM3072, t, src, p2, p3, m2, m3, mods);
    return cluster_launch(ctx, crt_slab12288_kernel<DIR, POST>, slabs, SMEM12288, t, src, p2, p3, m2, m3, mods);
}

/// The fused shape of a transform's plans (HC_SHAPE_L3072 or HC_SHAPE_L12288), or 0: both plan
/// lists are the specialised shapes with their compiled-in schedules and t has their extents.
int fused_shape(const hc_ntt_plan* plans2, const hc_ntt_plan* plans3, size_t r, const KView& t) {
    if (r == 0 || r > HC_MAX_MODS || (int64_t)r != t.n1) return 0;
    const int s2 = hc::plan_shape(plans2[0]), s3 = hc::plan_shape(plans3[0]);
    const bool f36864 = s2 == (HC_SHAPE_C12 | 0x100) && s3 == (HC_SHAPE_L3072 | 0x100) && t.n2 == 12 && t.n3 == 3072;
    const bool f49152 = s2 == (HC_SHAPE_C4 | 0x100) && s3 == (HC_SHAPE_L12288 | 0x100) && t.n2 == 4 && t.n3 == 12288;
    if (!f36864 && !f49152) return 0;
    for (size_t j = 1; j < r; j++)
        if (hc::plan_shape(plans2[j]) != s2 || hc::plan_shape(plans3[j]) != s3) return 0;
    if (t.n0 * t.n1 * CLUSTER > 0x7fffffff) return 0;
    return s3 & 0xff;
}

}  // namespace

namespace hc {

/// Whether the fused passes can run this transform: the plans are the fused shapes (fused_shape)
/// and the device runs the 12-CTA clusters of all three kernels of that shape.
bool crt_pass_ready(hc_context ctx, const hc_ntt_plan* plans2, const hc_ntt_plan* plans3, size_t r, const KView& t) {
    (void)ctx;
    const int shape3 = fused_shape(plans2, plans3, r, t);
    if (shape3 == HC_SHAPE_L3072)
        return cluster_ready(crt_slab3072_kernel<0, false>, SMEM3072) &&
               cluster_ready(crt_slab3072_kernel<1, false>, SMEM3072) &&
               cluster_ready(crt_slab3072_kernel<1, true>, SMEM3072);
    if (shape3 == HC_SHAPE_L12288)
        return cluster_ready(crt_slab12288_kernel<0, false>, SMEM12288) &&
               cluster_ready(crt_slab12288_kernel<1, false>, SMEM12288) &&
               cluster_ready(crt_slab12288_kernel<1, true>, SMEM12288);
    return false;
}

/// One fused half of a CRT transform over t [count, r, deg_L', deg_K] (dimension 3 contiguous):
/// dir 0 = ntt_mul along dimension 2 by m2, then along dimension 3 by m3 (reading the input from
/// src when given: the caller's copy folded into phase 1; src must not overlap t other than
/// exactly); dir 1 = intt along dimension 2, then along dimension 3, times m3 when `post`.
/// The caller checks crt_pass_ready first.
hc_status launch_crt_pass(hc_context ctx, int dir, const KView& t, const KView* src, const hc_ntt_plan* plans2,
                          const hc_ntt_plan* plans3, size_t r, const KView& m2, const KView& m3, bool post,
                          const KMods& mods) {
    const int shape3 = fused_shape(plans2, plans3, r, t);
    if (!shape3) return fail(HC_ERR_UNSUPPORTED, "fused CRT pass: plans are not a fused shape");
    PlanPtrs p2, p3;
    for (size_t j = 0; j < r; j++) {
        p2.p[j] = reinterpret_cast<const DevPlanHeader*>(plan_device(plans2[j]));
        p3.p[j] = reinterpret_cast<const DevPlanHeader*>(plan_device(plans3[j]));
    }
    const int64_t slabs = t.n0 * t.n1;
    if (slabs == 0) return HC_OK;
    const KView& s = src ? *src : t;
    if (dir == 0) return launch_shape<0, false>(ctx, shape3, slabs, t, s, p2, p3, m2, m3, mods);
    if (post) return launch_shape<1, true>(ctx, shape3, slabs, t, s, p2, p3, m2, m3, mods);
    return launch_shape<1, false>(ctx, shape3, slabs, t, s, p2, p3, m2, m3, mods);
}

}  // namespace hc
