/*
 * ringcuda.h — ring-level and BFV-level entry points of the GB300 backend.
 *
 * The reference runs its ring (cyclosubfield-dbfv/src/ring.rs) and BFV (src/bfv.rs) layers on top
 * of the HAL trait. These entry points are the same operations with the HAL call sequences fused
 * into few sm_103a kernels (base conversion, Galois permutation, key-switch inner product,
 * tensor product); results are bit-identical to the reference's call sequences over
 * `hal::cpu` on the same inputs. A Rust `hal::cuda` binding only needs include/halcuda.h; these
 * exist for callers that want the fused hot path, and for the batched/served forms.
 *
 * Layout: a batch of ring elements over an RNS base of r factors is a 4-D device tensor
 * [count, r, deg_L', deg_K] of Montgomery-form residues (src/ring.rs:3-13). RNS bases are lists
 * of factor indices into the context's prime list (`RNSBaseIndices`, src/ring.rs:132-134).
 * Key-switching keys with d digits over r_key factors are 4-D tensors [2 d, r_key, deg_L', deg_K]
 * (rows 2t, 2t+1 hold the two components of digit t; src/bfv.rs:56-64). Gadget digits are
 * passed as d (start, end) pairs of base positions. Plaintext moduli t are i128 values given as
 * (low, high) int64 words. Random numbers come from the reference's splitmix64 generator
 * (src/bfv.rs:880-886) whose 64-bit state the caller owns and which the call advances.
 *
 * Threads and streams: a ring (its table caches and its side streams) is used from one host thread
 * at a time; calls are asynchronous on the context's current stream (hc_context_set_stream), and
 * calls issued on different streams of one context may run concurrently on the GPU. Some calls
 * (hc_bfv_hom_mul) run independent parts on the ring's side stream, forked from and joined back
 * into the current stream, which a CUDA-graph capture of the call records as parallel paths.
 */
#ifndef RINGCUDA_H
#define RINGCUDA_H

#include "halcuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hc_ring_s* hc_ring;

/* RingContext::new (src/ring.rs:622-652): samples the initial base of log2_q_lo..log2_q_hi bits
 * and the extension pool, with NTT plans and CRT kernels per factor. Fields: "field_2",
 * "field_16", "field_18", "field_32", "field_192", "field_36864", "field_49152". */
hc_status hc_ring_create(hc_context ctx, const char* field, size_t log2_q_lo, size_t log2_q_hi, size_t t_bits,
                         hc_ring* out);
/* RingContext::new_raw (src/ring.rs:657-677): given primes, base conversions only. */
hc_status hc_ring_create_raw(hc_context ctx, const char* field, const int64_t* primes, size_t n, hc_ring* out);
hc_status hc_ring_destroy(hc_ring ring);
size_t hc_ring_num_factors(hc_ring ring);
int64_t hc_ring_prime(hc_ring ring, size_t idx);
size_t hc_ring_initial_len(hc_ring ring);
/* out[0] = n = deg_L, out[1] = deg_L', out[2] = deg_K */
hc_status hc_ring_dims(hc_ring ring, size_t out[3]);
hc_status hc_ring_modulus(hc_ring ring, size_t idx, hc_modulus* out);
/* RingContext::extension_rns_base_for (src/ring.rs:716-731) */
hc_status hc_ring_extension_base(hc_ring ring, const size_t* base, size_t r, size_t* out, size_t* out_len);
/* NTT-domain CRT kernels of one factor (src/ring.rs:1338-1415): kernel_L' | kernel_K |
 * inverse kernel_L' | inverse kernel_K, host output of 2 (deg_L' + deg_K) values. */
hc_status hc_ring_crt_kernels(hc_ring ring, size_t idx, int64_t* out);

/* pb_to_crt_tensor / crt_to_pb_tensor (src/ring.rs:1118-1161), in place; inputs bounded by 2p. */
hc_status hc_ring_pb_to_crt(hc_ring ring, hc_view data, const size_t* base, size_t r);
hc_status hc_ring_crt_to_pb(hc_ring ring, hc_view data, const size_t* base, size_t r);
/* bconv_tensors (src/ring.rs:1527-1535): src [count, rs, ...] -> dst [count, rd, ...]. Unlike the
 * reference, `src` is left unchanged. */
hc_status hc_ring_bconv(hc_ring ring, hc_view dst, const size_t* dst_base, size_t rd, hc_view src,
                        const size_t* src_base, size_t rs);
/* bconv_gadget_tensors (src/ring.rs:1566-1574): src [1, r, ...] -> dst [d, r, ...]; src unchanged. */
hc_status hc_ring_bconv_gadget(hc_ring ring, hc_view dst, hc_view src, const size_t* base, size_t r,
                               const size_t* digits, size_t d);
/* apply_galois (src/ring.rs:1183-1222), one gather pass. */
hc_status hc_ring_apply_galois(hc_ring ring, hc_view dst, hc_view src, const size_t* base, size_t r, uint64_t g);

/* ---------------------------------------------------------------- BFV (src/bfv.rs) */
/* gen_sk (:180-190): sk [1, r0, ...] over the initial base, CRT basis */
hc_status hc_bfv_gen_sk(hc_ring ring, uint64_t* rng_state, hc_view sk);
/* No counterpart in the reference (whose gen_sk, src/bfv.rs:180-190, is sparse with Hamming weight
 * 128): a secret key with every coefficient uniform in {-1, 0, 1}, coefficient j = (splitmix64
 * draw j mod 3) - 1, the distribution the benchmark's configuration names; CRT basis, initial
 * base, like hc_bfv_gen_sk. The kernels do not depend on the key's distribution. */
hc_status hc_bfv_gen_sk_uniform_ternary(hc_ring ring, uint64_t* rng_state, hc_view sk);
/* bfv_enc (:294-307): ptxt holds n i128 coefficients (2 words each); ct [2, r, ...] */
hc_status hc_bfv_enc(hc_ring ring, uint64_t* rng_state, const size_t* base, size_t r, const int64_t t[2],
                     const int64_t* ptxt, hc_view sk, double log2_alpha, hc_view ct);
/* gen_ksk (:433-458), gen_rk (:462-474), gen_gk (:479-491); keys [2 d, r, ...] */
hc_status hc_bfv_gen_ksk(hc_ring ring, uint64_t* rng_state, const size_t* base, size_t r, hc_view old_sk,
                         hc_view new_sk, const size_t* digits, size_t d, double log2_alpha, hc_view keys);
hc_status hc_bfv_gen_rk(hc_ring ring, uint64_t* rng_state, hc_view sk, const size_t* digits, size_t d,
                        double log2_alpha, hc_view keys);
hc_status hc_bfv_gen_gk(hc_ring ring, uint64_t* rng_state, hc_view sk, uint64_t g, const size_t* digits, size_t d,
                        double log2_alpha, hc_view keys);
/* log2_alpha_for_sigma (:165-167) */
double hc_bfv_log2_alpha_for_sigma(hc_ring ring, const size_t* base, size_t r, double sigma);
/* noisy_plaintext (:330-343): c0 + c1 s in period basis, out [1, r, ...] (decoding is host work) */
hc_status hc_bfv_noisy_plaintext(hc_ring ring, hc_view ct, const size_t* base, size_t r, hc_view sk, hc_view out);
/* key_switch (:533-556): c0 [1, r] CRT basis, c1 [1, r] period basis, keys over r_key >= r rows
 * (restricted on the fly) -> out [2, r] CRT basis */
hc_status hc_bfv_key_switch(hc_ring ring, hc_view c0_crt, hc_view c1_pb, const size_t* base, size_t r, hc_view keys,
                            const size_t* digits, size_t d, hc_view out);
/* lift_to_extended (:564-595): pb [count, r] (bound <= 2), crt optional (ptr NULL = absent)
 * -> out [count, r + ext] CRT basis */
hc_status hc_bfv_lift_to_extended(hc_ring ring, hc_view pb, hc_view crt, const size_t* base, size_t r, hc_view out);
/* rescale_to_base (:601-622): x [count, r + ext] period basis (modified) -> out [count, base_len] */
hc_status hc_bfv_rescale_to_base(hc_ring ring, hc_view x, const size_t* base, size_t r, size_t base_len,
                                 const int64_t t[2], hc_view out);
/* mod_switch_down (:628-662): x [count, r] period basis -> out [count, new_len] */
hc_status hc_bfv_mod_switch_down(hc_ring ring, hc_view x, const size_t* base, size_t r, size_t new_len, hc_view out);
/* bfv_hom_mul (:747-775): ct1, ct2 [2, r] CRT basis -> out [2, r] (CRT basis, or period basis
 * with bound 2 when period_output != 0). */
hc_status hc_bfv_hom_mul(hc_ring ring, const int64_t t[2], hc_view ct1, hc_view ct2, const size_t* base, size_t r,
                         hc_view rk, const size_t* digits, size_t d, int period_output, hc_view out);
/* bfv_hom_gal (:783-841): one Galois key per automorphism, gks [ngs * 2 d, r_key, ...]
 * -> out [ngs * 2, r, ...] CRT basis */
hc_status hc_bfv_hom_gal(hc_ring ring, hc_view ct, const size_t* base, size_t r, const uint64_t* gs, size_t ngs,
                         hc_view gks, const size_t* digits, size_t d, hc_view out);

/* bfv_hom_gal of B ciphertexts ct [2B, r] (CRT basis) under one automorphism g with its key
 * gk [2 d, r_key, ...] -> out [2B, r]; the batched form of hc_bfv_hom_gal with one element. */
hc_status hc_bfv_hom_gal_batch(hc_ring ring, hc_view ct, const size_t* base, size_t r, uint64_t g, hc_view gk,
                               const size_t* digits, size_t d, hc_view out);

/* Batched CRT transforms of many ring elements of different fields and RNS lengths in one
 * persistent launch. Each item is a tensor of elements of one ring over one base; per element
 * and factor ("slab") the batch runs, as `ops` says, pb_to_crt (src/ring.rs:1118-1138), a
 * Montgomery product with the item's operand (hal_mul_mont64, src/hal/cpu.rs:823-836) and
 * crt_to_pb (:1140-1161), in place and bit-identical to those calls made one by one. The batch
 * keeps device pointers to the items' tensors and to the rings' tables: both must outlive it.
 * Running it issues, per shape class of its slabs (each field's specialised line and column
 * shapes; one class for the rest), a counter reset and one persistent kernel on the context's
 * stream (graph-capturable). */
#define HC_CRT_FORWARD 1 /* period basis -> CRT basis (input bound 2) */
#define HC_CRT_MUL 2     /* Montgomery product with `op` (CRT basis) */
#define HC_CRT_INVERSE 4 /* CRT basis -> period basis */
#define HC_CRT_ONE_LAUNCH 8 /* with the above: every slab in one persistent launch, one launch shape
                             * (default: one launch per shape class, each with its own shape) */
typedef struct hc_crt_batch_s* hc_crt_batch;
typedef struct {
    hc_ring ring;
    hc_view data;        /* [count, r, deg_L', deg_K], transformed in place */
    hc_view op;          /* [count | 1, r, deg_L', deg_K] for HC_CRT_MUL, else ptr NULL */
    const size_t* base;  /* r factor indices of the ring */
    size_t r;
} hc_crt_item;
/* Launch shape of the persistent kernel: threads per CTA (32..256), CTAs per SM, and 2^logv
 * columns per dimension-2 tile (logv 0..6). Each shape class has its own; set_launch sets all
 * of them, get_launch and tune report that of the class with the most residues. */
typedef struct {
    int threads;
    int ctas_per_sm;
    int logv;
} hc_crt_launch;
hc_status hc_crt_batch_create(hc_context ctx, const hc_crt_item* items, size_t n, int ops, hc_crt_batch* out);
hc_status hc_crt_batch_run(hc_crt_batch b);
/* Autotuner: per shape class, times every launch shape of a fixed candidate set on a scratch copy
 * of (a sample of) the class's slabs - the transforms are data-oblivious - and keeps the fastest;
 * the choice is remembered for classes of the same composition. Synchronises; not during stream
 * capture. */
hc_status hc_crt_batch_tune(hc_crt_batch b, int reps, hc_crt_launch* chosen);
hc_status hc_crt_batch_set_launch(hc_crt_batch b, const hc_crt_launch* l);
hc_status hc_crt_batch_get_launch(hc_crt_batch b, hc_crt_launch* out);
size_t hc_crt_batch_num_slabs(hc_crt_batch b);
hc_status hc_crt_batch_destroy(hc_crt_batch b);

/* Galois keysets: the device-side replacement of the reference's key offloading
 * (KeySwitchKey::offload_to_disk, src/bfv.rs:95-116, and the mmap keystore, src/keystore.rs:87-119).
 * Keys of one gadget split (d digits over r_key factors, each [2 d, r_key, deg_L', deg_K]) stay in
 * HBM while the resident bytes fit `hbm_budget_bytes`; further keys are moved to pinned host memory
 * and copied into one of two device slots right before their key switch, on a separate copy
 * stream, so that the next key's copy overlaps the current key switch. */
typedef struct hc_keyset_s* hc_keyset;
hc_status hc_keyset_create(hc_ring ring, const size_t* digits, size_t d, size_t r_key, size_t hbm_budget_bytes,
                           hc_keyset* out);
/* Adds (copies) the Galois key of automorphism g; `key` is a contiguous device tensor. */
hc_status hc_keyset_add(hc_keyset ks, uint64_t g, hc_view key);
hc_status hc_keyset_stats(hc_keyset ks, size_t* resident, size_t* streamed, uint64_t* streamed_keys,
                          uint64_t* streamed_bytes);
hc_status hc_keyset_destroy(hc_keyset ks);
/* bfv_hom_gal (src/bfv.rs:783-841) with the keys of a keyset: ct [2, r] CRT -> out [ngs * 2, r] */
hc_status hc_bfv_hom_gal_keyset(hc_ring ring, hc_view ct, const size_t* base, size_t r, const uint64_t* gs, size_t ngs,
                                hc_keyset ks, hc_view out);
/* bfv_hom_gal (src/bfv.rs:783-841) of B ciphertexts ct [2B, r] (rows 2i, 2i + 1) under one
 * automorphism g whose key comes from a keyset (streamed in when it is over the HBM budget):
 * one gadget decomposition and one key-switch launch for the batch -> out [2B, r]. A keyset
 * without a key for g is refused (HC_ERR_ARG) before any work is queued. */
hc_status hc_bfv_hom_gal_batch_keyset(hc_ring ring, hc_view ct, const size_t* base, size_t r, uint64_t g, hc_keyset ks,
                                      hc_view out);
/* hom_cyclic_transform_dbfv (src/bootstrap/homcrt.rs:369-429): the dBFV ciphertext ct [2 d, r]
 * (CRT basis, almost reduced) is mapped to sum_i coeffs[i] sigma_g^i(ct) by baby-step giant-step:
 * the baby steps share one gadget decomposition per digit, every giant step applies one unhoisted
 * automorphism; coefficients are L' elements (len x deg_L' i128 values as (low, high) words),
 * decomposed into balanced digits of base b = 2^log2_b, t = 2^log2_t. out has 2 * digits rows
 * (digits = ceil(log2_t / log2_b)); *out_rows receives the rows written. */
hc_status hc_dbfv_hom_cyclic_transform(hc_ring ring, size_t log2_b, size_t log2_t, uint64_t g, const int64_t* coeffs,
                                       size_t len, hc_view ct, const size_t* base, size_t r, hc_keyset ks, hc_view out,
                                       size_t* out_rows);

/* dBFV reduction path (src/dbfv.rs:661-1143): t = 2^log2_t in digits of b = 2^log2_b.
 * dbfv_reduce (:968-1032): ct [2 d, r] period basis with entries bounded by `bound` p -> out (at
 * least 2 digits rows; *out_rows written), every digit reduced modulo b Delta with its overflow
 * carried into the next digit (split_overflow, :891-950). */
hc_status hc_dbfv_reduce(hc_ring ring, size_t log2_b, size_t log2_t, hc_view ct, const size_t* base, size_t r,
                         uint64_t bound, hc_view out, size_t* out_rows);
/* dbfv_enc (:661-689): n i128 plaintext coefficients -> out [2 digits, r] CRT basis */
hc_status hc_dbfv_enc(hc_ring ring, uint64_t* rng_state, size_t log2_b, size_t log2_t, const size_t* base, size_t r,
                      const int64_t* ptxt, hc_view sk, double log2_alpha, hc_view out);
/* dbfv_hom_mul (:1034-1059, digit convolution :1081-1143): lhs [2 d1, r], rhs [2 d2, r] period
 * basis -> out (CRT basis, or period basis when period_output), *out_rows = 2 min(digits, d1 + d2 - 1) */
hc_status hc_dbfv_hom_mul(hc_ring ring, size_t log2_b, size_t log2_t, hc_view lhs, hc_view rhs, const size_t* base,
                          size_t r, hc_view rk, const size_t* digits, size_t d, int period_output, hc_view out,
                          size_t* out_rows);

/* No counterpart in the reference (its CPU backend allocates freely): hc_bfv_key_switch with the
 * same arguments and the same result, for callers that cannot allocate device memory - a host
 * whose HBM is handed out by its own arena or budget, or a code path where cudaMalloc / cudaFree
 * are not permitted or would synchronise the device at the wrong moment. It allocates nothing:
 * the gadget digits are kept in a static device array of 32 MiB (2^22 i64 words) that every GPU
 * loading this library holds until the process exits.
 *  - d x r x deg_L' x deg_K must be at most 2^22 (field_36864: d r <= 113), else
 *    HC_ERR_UNSUPPORTED.
 *  - The ring's tables for this base and digit split must exist: any key-switching call with the
 *    same base and digit split builds them (hc_bfv_key_switch, the relinearisation of
 *    hc_bfv_hom_mul, hc_bfv_hom_gal); without them the call fails with HC_ERR_ARG.
 *  - The first call on a device looks up the array's device address (cudaGetSymbolAddress, with
 *    that device current); make that first call before any stream capture. The address is kept
 *    for the life of the process: a device reset (cudaDeviceReset) invalidates it, as it
 *    invalidates every device object of this library, so no call may follow a reset.
 *  - All calls share the one array: calls whose kernels may overlap on the GPU (other streams,
 *    other contexts on the same device) race and corrupt each other's results. */
hc_status hc_bfv_key_switch_noalloc(hc_ring ring, hc_view c0_crt, hc_view c1_pb, const size_t* base, size_t r,
                                    hc_view keys, const size_t* digits, size_t d, hc_view out);

#ifdef __cplusplus
}
#endif

#endif /* RINGCUDA_H */
