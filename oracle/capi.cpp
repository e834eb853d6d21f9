// ORACLE — test infrastructure only. The extern "C" surface through which tests/ (ctypes)
// drive the CPU restatement: one entry per Backend method (src/hal/mod.rs:108-350) over strided
// views, and ring/BFV entry points over contiguous [count, r, deg_L', deg_K] arrays.
#include <cstdio>
#include <cstring>

#include "dbfv.hpp"

using namespace oracle;

extern "C" {

struct or_view {
    void* ptr;
    int64_t shape[4];
    int64_t strides[4];
};
}

namespace {
thread_local std::string g_last_error;

template <typename T>
View<T> to_view(const or_view* v) {
    View<T> r;
    r.ptr = (T*)v->ptr;
    for (int d = 0; d < 4; d++) {
        r.shape[d] = (size_t)v->shape[d];
        r.strides[d] = (size_t)v->strides[d];
    }
    ORACLE_ASSERT(r.strides[3] == 1 || r.shape[3] <= 1, "dimension 3 must be contiguous");
    return r;
}

Mods mods_from(const int64_t* primes, size_t n) {
    Mods m;
    for (size_t i = 0; i < n; i++) m.push_back(MontgomeryModulus::create(primes[i]));
    return m;
}

template <typename F>
int guarded(F f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return 1;
    }
}

const CpuBackend BE;

struct BfvHandle {
    std::unique_ptr<RingContext> ring;
};

Base base_from(const size_t* b, size_t r) { return Base(b, b + r); }

RingEls els_from(const RingContext& ring, const int64_t* data, size_t count, const Base& base, Basis basis) {
    RingEls e = ring.allocate_in_basis(count, base, basis);
    std::memcpy(e.data.data.data(), data, e.data.data.size() * sizeof(int64_t));
    return e;
}
void els_to(const RingEls& e, int64_t* out) { std::memcpy(out, e.data.data.data(), e.data.data.size() * sizeof(int64_t)); }

Digits digits_from(const size_t* d, size_t n) {
    Digits r;
    for (size_t i = 0; i < n; i++) r.push_back({d[2 * i], d[2 * i + 1]});
    return r;
}

// keys: [d, 2, r_key, dl, dk] contiguous
KeySwitchKey key_from(const RingContext& ring, const int64_t* keys, size_t d, const Digits& digits, size_t r_key) {
    KeySwitchKey k;
    k.digits = digits;
    Base base;
    for (size_t i = 0; i < r_key; i++) base.push_back(i);
    size_t per = 2 * r_key * ring.n();
    for (size_t i = 0; i < d; i++) k.keys.push_back(els_from(ring, keys + i * per, 2, base, Basis::CRTBasis));
    return k;
}
void key_to(const KeySwitchKey& k, int64_t* out) {
    size_t off = 0;
    for (auto& e : k.keys) {
        els_to(e, out + off);
        off += e.data.data.size();
    }
}
}  // namespace

extern "C" {

const char* or_last_error() { return g_last_error.c_str(); }

// ---------------- scalar arithmetic probes ----------------
int or_mont_constants(int64_t prime, int64_t* out4) {
    return guarded([&] {
        MontgomeryModulus m = MontgomeryModulus::create(prime);
        out4[0] = m.N, out4[1] = m.neg_inv_N, out4[2] = m.R_sqr_mod_N, out4[3] = m.R_cbe_mod_N;
    });
}
int or_barrett(int64_t value, int64_t n, const int64_t* xs, size_t len, int64_t* out, int64_t* zu) {
    return guarded([&] {
        BarrettMul b = BarrettMul::create(value, n);
        zu[0] = b.z, zu[1] = b.u;
        for (size_t i = 0; i < len; i++) out[i] = b.mul(xs[i], n);
    });
}
/// out: red128, double_red128, to_mont128 of each i128 input (given as lo/hi pairs), to_mont64 of lo
int or_mont_ops(int64_t prime, const int64_t* x128, size_t len, int64_t* out) {
    return guarded([&] {
        MontgomeryModulus m = MontgomeryModulus::create(prime);
        for (size_t i = 0; i < len; i++) {
            i128 x = (i128)(((u128)(uint64_t)x128[2 * i + 1] << 64) | (uint64_t)x128[2 * i]);
            out[4 * i + 0] = m.red128(x);
            out[4 * i + 1] = m.double_red128(x);
            out[4 * i + 2] = m.to_mont128(x);
            out[4 * i + 3] = m.to_mont64((int64_t)x);
        }
    });
}
/// Single-factor transform on a contiguous line (src/hal/ntt.rs:686-694 test helpers).
int or_factor_ntt(int64_t q, size_t len, int64_t* data, int inverse, int reduce_output, int64_t in_bound_lo,
                  uint64_t* out_bound) {
    return guarded([&] {
        LazyFactorNTT f = LazyFactorNTT::create(q, len);
        u128 b = inverse ? f.backward(data, 1, 1, (u128)in_bound_lo, false, BarrettMul{0, 0})
                         : f.forward(data, 1, 1, (u128)in_bound_lo, reduce_output != 0);
        *out_bound = (uint64_t)b;
    });
}
int or_plan_apply(int64_t q, const size_t* shape, size_t k, int64_t* data, size_t elem_stride, size_t vec_len,
                  int inverse, int reduce_output) {
    return guarded([&] {
        CpuNTTPlan p = CpuNTTPlan::create(q, std::vector<size_t>(shape, shape + k));
        p.apply(data, elem_stride, vec_len, inverse != 0, reduce_output != 0);
    });
}
int64_t or_find_root_of_unity(int64_t q, size_t n) { return find_root_of_unity(q, n); }

// ---------------- Backend methods over strided views ----------------
int or_assign(const or_view* d, const or_view* s) { return guarded([&] { BE.hal_assign(to_view<int64_t>(d), to_view<int64_t>(s)); }); }
int or_assign_narrow(const or_view* d, const or_view* s) {
    return guarded([&] { BE.hal_assign_narrow(to_view<int64_t>(d), to_view<i128>(s)); });
}
int or_assign_i128(const or_view* d, const or_view* s) { return guarded([&] { BE.hal_assign_i128(to_view<i128>(d), to_view<i128>(s)); }); }
int or_add_i64(const or_view* d, const or_view* s) { return guarded([&] { BE.hal_add_i64(to_view<int64_t>(d), to_view<int64_t>(s)); }); }
int or_sub_i64(const or_view* d, const or_view* s) { return guarded([&] { BE.hal_sub_i64(to_view<int64_t>(d), to_view<int64_t>(s)); }); }
int or_add_i128(const or_view* d, const or_view* s) { return guarded([&] { BE.hal_add_i128(to_view<i128>(d), to_view<i128>(s)); }); }
int or_fma_i64(const or_view* d, const or_view* l, const or_view* r) {
    return guarded([&] { BE.hal_fma_i64(to_view<i128>(d), to_view<int64_t>(l), to_view<int64_t>(r)); });
}
int or_mul_i64(const or_view* d, const or_view* l, const or_view* r) {
    return guarded([&] { BE.hal_mul_i64(to_view<i128>(d), to_view<int64_t>(l), to_view<int64_t>(r)); });
}
int or_inner_product_i64(const or_view* d, const or_view* l, const or_view* r, size_t terms) {
    return guarded([&] {
        std::vector<V64> lv, rv;
        for (size_t t = 0; t < terms; t++) lv.push_back(to_view<int64_t>(&l[t])), rv.push_back(to_view<int64_t>(&r[t]));
        BE.hal_inner_product_i64(to_view<i128>(d), lv, rv);
    });
}
int or_matmul_i64(const or_view* d, const or_view* l, const or_view* r) {
    return guarded([&] { BE.hal_matmul_i64(to_view<i128>(d), to_view<int64_t>(l), to_view<int64_t>(r)); });
}
int or_mul_mont64(const or_view* d, const or_view* s, const int64_t* primes, size_t n) {
    return guarded([&] { BE.hal_mul_mont64(to_view<int64_t>(d), to_view<int64_t>(s), mods_from(primes, n)); });
}
/// kind: 0 add_red_mont64_double, 1 red_mont64_double, 2 add_red_mont64, 3 red_mont64, 4 i128_to_mont64
int or_red128(int kind, const or_view* d, const or_view* s, const int64_t* primes, size_t n) {
    return guarded([&] {
        Mods m = mods_from(primes, n);
        V64 dv = to_view<int64_t>(d);
        V128 sv = to_view<i128>(s);
        switch (kind) {
            case 0: BE.hal_add_red_mont64_double(dv, sv, m); break;
            case 1: BE.hal_red_mont64_double(dv, sv, m); break;
            case 2: BE.hal_add_red_mont64(dv, sv, m); break;
            case 3: BE.hal_red_mont64(dv, sv, m); break;
            case 4: BE.hal_i128_to_mont64(dv, sv, m); break;
            default: fail("unknown reduction kind");
        }
    });
}
int or_i64_to_mont64(const or_view* d, const int64_t* primes, size_t n) {
    return guarded([&] { BE.hal_i64_to_mont64(to_view<int64_t>(d), mods_from(primes, n)); });
}
/// mode: 0 ntt, 1 intt, 2 ntt_mul (mul view used). One plan per prime, all with `shape`.
int or_ntt_dim(const or_view* d, const int64_t* primes, size_t n, const size_t* shape, size_t k, int dim, int mode,
               const or_view* mul) {
    return guarded([&] {
        std::vector<CpuNTTPlan> plans;
        for (size_t i = 0; i < n; i++) plans.push_back(CpuNTTPlan::create(primes[i], std::vector<size_t>(shape, shape + k)));
        Plans pp;
        for (auto& p : plans) pp.push_back(&p);
        DataDim dd = dim == 2 ? DataDim::Dim2 : DataDim::Dim3;
        V64 dv = to_view<int64_t>(d);
        if (mode == 0) BE.hal_ntt_mont64_dim(dv, pp, dd);
        else if (mode == 1) BE.hal_intt_mont64_dim(dv, pp, dd);
        else BE.hal_ntt_mul_mont64_dim(dv, pp, dd, to_view<int64_t>(mul), mods_from(primes, n));
    });
}
int or_bconv_correct_mont64(const or_view* d, const or_view* l, const or_view* r, const int64_t* primes, size_t n,
                            size_t shift) {
    return guarded([&] {
        BE.hal_bconv_correct_mont64(to_view<int64_t>(d), to_view<i128>(l), to_view<int64_t>(r), mods_from(primes, n),
                                    shift);
    });
}
int or_bconv_correct_pow2(const or_view* d, const or_view* s, int64_t f0, int64_t f1, size_t shift, size_t log2m) {
    return guarded([&] { BE.hal_bconv_correct_pow2(to_view<int64_t>(d), to_view<i128>(s), f0, f1, shift, log2m); });
}
int or_bconv_correct_pow2_wide(const or_view* d, const or_view* s, int64_t f0lo, int64_t f0hi, int64_t f1lo,
                               int64_t f1hi, size_t shift, size_t log2m) {
    return guarded([&] {
        i128 f0 = (i128)(((u128)(uint64_t)f0hi << 64) | (uint64_t)f0lo);
        i128 f1 = (i128)(((u128)(uint64_t)f1hi << 64) | (uint64_t)f1lo);
        BE.hal_bconv_correct_pow2_wide(to_view<int64_t>(d), to_view<i128>(s), f0, f1, shift, log2m);
    });
}
int or_create_permutation(const size_t* shape, const size_t* shifts, size_t k, uint32_t* out_perm) {
    return guarded([&] {
        CpuPermutationPlan p =
            BE.hal_create_permutation(std::vector<size_t>(shape, shape + k), std::vector<size_t>(shifts, shifts + k));
        std::memcpy(out_perm, p.perm.data(), p.len * sizeof(uint32_t));
    });
}
int or_permute(const or_view* d, const or_view* s, const size_t* shape, const size_t* shifts, size_t k, int dim) {
    return guarded([&] {
        CpuPermutationPlan p =
            BE.hal_create_permutation(std::vector<size_t>(shape, shape + k), std::vector<size_t>(shifts, shifts + k));
        BE.hal_permute(to_view<int64_t>(d), to_view<int64_t>(s), p, dim == 2 ? DataDim::Dim2 : DataDim::Dim3);
    });
}

// ---------------- field ----------------
/// Writes m, deg_l, deg_lprime, deg_k, #lprime factors, #factors, rou_order; orders/gens after.
int or_field_info(const char* name, uint64_t* out, size_t cap) {
    return guarded([&] {
        FieldDescriptor f = field_by_name(name);
        std::vector<uint64_t> v{f.m, f.deg_l, f.deg_lprime, f.deg_k, f.lprime_factor_count, f.lq_cyclic.size(),
                                f.rou_order(), f.gal_ml.size()};
        for (auto& c : f.lq_cyclic) v.push_back(c.second);
        for (auto& c : f.lq_cyclic) v.push_back(c.first);
        ORACLE_ASSERT(v.size() <= cap, "field info buffer");
        std::memcpy(out, v.data(), v.size() * sizeof(uint64_t));
    });
}
int or_gal_to_shift(const char* name, uint64_t g, int64_t* out) {
    return guarded([&] {
        FieldDescriptor f = field_by_name(name);
        std::vector<int64_t> s = f.gal_to_shift(g);
        std::memcpy(out, s.data(), s.size() * sizeof(int64_t));
    });
}

// ---------------- ring ----------------
void* or_ring_create(const char* field, size_t lo, size_t hi, size_t t_bits) {
    void* res = nullptr;
    if (guarded([&] {
            auto* h = new BfvHandle();
            h->ring = RingContext::create(field_by_name(field), lo, hi, t_bits);
            res = h;
        }))
        return nullptr;
    return res;
}
void* or_ring_create_raw(const char* field, const int64_t* primes, size_t n) {
    void* res = nullptr;
    if (guarded([&] {
            auto* h = new BfvHandle();
            h->ring = RingContext::create_raw(field_by_name(field), std::vector<int64_t>(primes, primes + n));
            res = h;
        }))
        return nullptr;
    return res;
}
void or_ring_free(void* h) { delete (BfvHandle*)h; }
size_t or_ring_num_factors(void* h) { return ((BfvHandle*)h)->ring->rns_factors.size(); }
size_t or_ring_initial_len(void* h) { return ((BfvHandle*)h)->ring->initial_rns_base_len; }
int64_t or_ring_prime(void* h, size_t i) { return ((BfvHandle*)h)->ring->rns_factors[i].p; }
int or_ring_extension_base(void* h, const size_t* base, size_t r, size_t* out, size_t* out_len) {
    return guarded([&] {
        Base e = ((BfvHandle*)h)->ring->extension_rns_base_for(base_from(base, r));
        std::memcpy(out, e.data(), e.size() * sizeof(size_t));
        *out_len = e.size();
    });
}
/// out: crt_kernel_lprime | crt_kernel_k | inv_crt_kernel_lprime | inv_crt_kernel_k for the factor
int or_ring_kernels(void* h, size_t idx, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        TransformCache& c = ring.transform_cache_for(Base{idx});
        size_t dl = ring.field.deg_lprime, dk = ring.field.deg_k;
        std::memcpy(out, c.crt_kernel_lprime.data.data(), dl * 8);
        std::memcpy(out + dl, c.crt_kernel_k.data.data(), dk * 8);
        std::memcpy(out + dl + dk, c.inv_crt_kernel_lprime.data.data(), dl * 8);
        std::memcpy(out + 2 * dl + dk, c.inv_crt_kernel_k.data.data(), dk * 8);
    });
}
int or_ring_pb_to_crt(void* h, int64_t* data, size_t count, const size_t* base, size_t r, int inverse) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Base b = base_from(base, r);
        V64 v{data, Shape{count, r, ring.field.deg_lprime, ring.field.deg_k}, Shape{}};
        v.strides = strides_for(v.shape);
        if (inverse) ring.crt_to_pb_tensor(v, b);
        else ring.pb_to_crt_tensor(v, b);
    });
}
/// Tensors are [count, r, 1, ncoef] (base conversion is pointwise over the coefficients).
int or_ring_bconv(void* h, int64_t* dst, const size_t* dst_base, size_t rd, int64_t* src, const size_t* src_base,
                  size_t rs, size_t count, size_t ncoef) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Shape ds{count, rd, 1, ncoef}, ss{count, rs, 1, ncoef};
        ring.bconv_tensors(V64{dst, ds, strides_for(ds)}, base_from(dst_base, rd), V64{src, ss, strides_for(ss)},
                           base_from(src_base, rs));
    });
}
int or_ring_bconv_gadget(void* h, int64_t* dst, int64_t* src, const size_t* base, size_t r, const size_t* digits,
                         size_t d, size_t ncoef) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Shape ds{d, r, 1, ncoef}, ss{1, r, 1, ncoef};
        ring.bconv_gadget_tensors(V64{dst, ds, strides_for(ds)}, V64{src, ss, strides_for(ss)}, base_from(base, r),
                                  digits_from(digits, d));
    });
}
int or_ring_apply_galois(void* h, int64_t* dst, const int64_t* src, size_t count, const size_t* base, size_t r,
                         uint64_t g) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Base b = base_from(base, r);
        RingEls s = els_from(ring, src, count, b, Basis::CRTBasis);
        RingEls dd = ring.allocate_in_basis(count, b, Basis::CRTBasis);
        ring.apply_galois(dd, as_view(s), g);
        els_to(dd, dst);
    });
}

// ---------------- BFV ----------------
double or_bfv_log2_alpha_for_sigma(void* h, const size_t* base, size_t r, double sigma) {
    RingContext& ring = *((BfvHandle*)h)->ring;
    uint64_t st = 0;
    return Bfv(ring, &st).log2_alpha_for_sigma(base_from(base, r), sigma);
}
int or_bfv_gen_sk(void* h, uint64_t* state, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        els_to(Bfv(ring, state).gen_sk(), out);
    });
}
/// ptxt: n i128 values as (lo, hi) int64 pairs; t as (lo, hi)
int or_bfv_enc(void* h, uint64_t* state, const size_t* base, size_t r, int64_t t_lo, int64_t t_hi, const int64_t* ptxt,
               const int64_t* sk, double log2_alpha, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        i128 t = (i128)(((u128)(uint64_t)t_hi << 64) | (uint64_t)t_lo);
        std::vector<i128> m;
        for (size_t i = 0; i < ring.n(); i++) m.push_back((i128)(((u128)(uint64_t)ptxt[2 * i + 1] << 64) | (uint64_t)ptxt[2 * i]));
        RingEls s = els_from(ring, sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        els_to(Bfv(ring, state).bfv_enc(base_from(base, r), t, m, s, log2_alpha), out);
    });
}
int or_bfv_gen_rk(void* h, uint64_t* state, const int64_t* sk, const size_t* digits, size_t d, double log2_alpha,
                  int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        RingEls s = els_from(ring, sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        key_to(Bfv(ring, state).gen_rk(s, digits_from(digits, d), log2_alpha), out);
    });
}
/// old_sk / new_sk over the initial base; keys over `base`
int or_bfv_gen_ksk(void* h, uint64_t* state, const size_t* base, size_t r, const int64_t* old_sk,
                   const int64_t* new_sk, const size_t* digits, size_t d, double log2_alpha, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        RingEls o = els_from(ring, old_sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        RingEls n = els_from(ring, new_sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        key_to(Bfv(ring, state).gen_ksk(base_from(base, r), o, n, digits_from(digits, d), log2_alpha), out);
    });
}
int or_bfv_gen_gk(void* h, uint64_t* state, const int64_t* sk, uint64_t g, const size_t* digits, size_t d,
                  double log2_alpha, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        RingEls s = els_from(ring, sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        key_to(Bfv(ring, state).gen_gk(s, g, digits_from(digits, d), log2_alpha), out);
    });
}
int or_bfv_noisy_plaintext(void* h, const int64_t* ct, const size_t* base, size_t r, const int64_t* sk, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        RingEls c = els_from(ring, ct, 2, base_from(base, r), Basis::CRTBasis);
        RingEls s = els_from(ring, sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        els_to(Bfv(ring, &st).noisy_plaintext(as_view(c), s), out);
    });
}
/// keys: [d, 2, r_key, dl, dk]; output [2, r, dl, dk]
int or_bfv_hom_mul(void* h, int64_t t_lo, int64_t t_hi, const int64_t* ct1, const int64_t* ct2, const size_t* base,
                   size_t r, const int64_t* keys, const size_t* digits, size_t d, size_t r_key, int period_output,
                   int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        i128 t = (i128)(((u128)(uint64_t)t_hi << 64) | (uint64_t)t_lo);
        Base b = base_from(base, r);
        RingEls a = els_from(ring, ct1, 2, b, Basis::CRTBasis);
        RingEls c = els_from(ring, ct2, 2, b, Basis::CRTBasis);
        KeySwitchKey rk = key_from(ring, keys, d, digits_from(digits, d), r_key);
        els_to(Bfv(ring, &st).bfv_hom_mul(t, a, c, rk, period_output ? Basis::PeriodBasis : Basis::CRTBasis), out);
    });
}
/// keys: [ngs, d, 2, r_key, dl, dk]; output [ngs, 2, r, dl, dk]
int or_bfv_hom_gal(void* h, const int64_t* ct, const size_t* base, size_t r, const uint64_t* gs, size_t ngs,
                   const int64_t* keys, const size_t* digits, size_t d, size_t r_key, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        Base b = base_from(base, r);
        RingEls c = els_from(ring, ct, 2, b, Basis::CRTBasis);
        std::vector<KeySwitchKey> ks;
        size_t per = d * 2 * r_key * ring.n();
        for (size_t i = 0; i < ngs; i++) ks.push_back(key_from(ring, keys + i * per, d, digits_from(digits, d), r_key));
        std::vector<const KeySwitchKey*> kp;
        for (auto& k : ks) kp.push_back(&k);
        auto res = Bfv(ring, &st).bfv_hom_gal(as_view(c), std::vector<uint64_t>(gs, gs + ngs), kp);
        size_t off = 0;
        for (auto& e : res) {
            els_to(e, out + off);
            off += e.data.data.size();
        }
    });
}
/// dbfv_enc (src/dbfv.rs:661-689): out [2 digits, r] CRT basis
int or_dbfv_enc(void* h, uint64_t* state, size_t log2_b, size_t log2_t, const size_t* base, size_t r,
                const int64_t* ptxt, const int64_t* sk, double log2_alpha, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Bfv bfv(ring, state);
        RingEls s = els_from(ring, sk, 1, ring.initial_rns_base(), Basis::CRTBasis);
        std::vector<i128> m(ring.n());
        for (size_t i = 0; i < m.size(); i++) m[i] = (i128)(((u128)(uint64_t)ptxt[2 * i + 1] << 64) | (uint64_t)ptxt[2 * i]);
        els_to(dbfv_enc(ring, bfv, DBFVModulus{log2_b, log2_t}, base_from(base, r), m, s, log2_alpha), out);
    });
}
/// dbfv_reduce (src/dbfv.rs:968-1032): ct [2 d, r] period basis with entries bounded by
/// `bound` p -> out [2 digits, r] period basis (*out_rows rows)
int or_dbfv_reduce(void* h, size_t log2_b, size_t log2_t, const int64_t* ct, size_t d, const size_t* base, size_t r,
                   uint64_t bound, int64_t* out, size_t* out_rows) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        RingEls c = els_from(ring, ct, 2 * d, base_from(base, r), Basis::PeriodBasis);
        c.bound = bound;
        RingEls res = dbfv_reduce(ring, DBFVModulus{log2_b, log2_t}, as_view(c));
        els_to(res, out);
        *out_rows = res.count();
    });
}
/// dbfv_hom_mul (src/dbfv.rs:1034-1059): lhs [2 d1, r], rhs [2 d2, r] period basis -> out
/// (CRT basis, or period basis when period_output) with *out_rows rows
int or_dbfv_hom_mul(void* h, size_t log2_b, size_t log2_t, const int64_t* lhs, size_t d1, const int64_t* rhs, size_t d2,
                    const size_t* base, size_t r, const int64_t* rk, const size_t* digits, size_t dk, size_t r_key,
                    int period_output, int64_t* out, size_t* out_rows) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        Bfv bfv(ring, &st);
        Base b = base_from(base, r);
        RingEls l = els_from(ring, lhs, 2 * d1, b, Basis::PeriodBasis), rr = els_from(ring, rhs, 2 * d2, b, Basis::PeriodBasis);
        KeySwitchKey k = key_from(ring, rk, dk, digits_from(digits, dk), r_key);
        RingEls res = dbfv_hom_mul(ring, bfv, DBFVModulus{log2_b, log2_t}, as_view(l), as_view(rr), k,
                                   period_output ? Basis::PeriodBasis : Basis::CRTBasis);
        els_to(res, out);
        *out_rows = res.count();
    });
}
/// lprime_element_tensor (src/ring.rs:1227-1250): deg_L' i128 coefficients (low, high words)
/// -> out [1, r, deg_L', 1] CRT basis, Montgomery form
int or_ring_lprime_element_tensor(void* h, const size_t* base, size_t r, const int64_t* coeffs, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        std::vector<i128> c(ring.field.deg_lprime);
        for (size_t k = 0; k < c.size(); k++)
            c[k] = (i128)(((u128)(uint64_t)coeffs[2 * k + 1] << 64) | (uint64_t)coeffs[2 * k]);
        Tensor<int64_t> t = ring.lprime_element_tensor(base_from(base, r), c);
        std::memcpy(out, t.data.data(), t.data.size() * sizeof(int64_t));
    });
}
/// hom_cyclic_transform_dbfv (src/bootstrap/homcrt.rs:369-429): ct [2 d_ct, r] CRT basis;
/// coeffs: len L' elements of deg_L' i128 coefficients as (low, high) int64 words; ngk Galois
/// keys stacked [ngk * 2 dk, r_key, ...] with their automorphisms gk_g. out receives the result
/// (at most 2 * digits rows), *out_rows its row count.
int or_dbfv_hom_cyclic_transform(void* h, size_t log2_b, size_t log2_t, uint64_t g, const int64_t* coeffs, size_t len,
                                 const int64_t* ct, size_t d_ct, const size_t* base, size_t r, const int64_t* gks,
                                 const uint64_t* gk_g, size_t ngk, const size_t* digits, size_t dk, size_t r_key,
                                 int64_t* out, size_t* out_rows) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Base b = base_from(base, r);
        RingEls c = els_from(ring, ct, 2 * d_ct, b, Basis::CRTBasis);
        std::vector<KeySwitchKey> ks;
        size_t per = dk * 2 * r_key * ring.n();
        for (size_t i = 0; i < ngk; i++) ks.push_back(key_from(ring, gks + i * per, dk, digits_from(digits, dk), r_key));
        auto key_for = [&](uint64_t gg) -> const KeySwitchKey* {
            for (size_t i = 0; i < ngk; i++)
                if (gk_g[i] == gg) return &ks[i];
            ORACLE_ASSERT(false, "missing galois key");
            return nullptr;
        };
        const size_t dl = ring.field.deg_lprime;
        std::vector<std::vector<i128>> cf(len, std::vector<i128>(dl));
        for (size_t i = 0; i < len; i++)
            for (size_t k = 0; k < dl; k++) {
                const int64_t* w = coeffs + 2 * (i * dl + k);
                cf[i][k] = (i128)(((u128)(uint64_t)w[1] << 64) | (uint64_t)w[0]);
            }
        RingEls res = hom_cyclic_transform_dbfv(ring, DBFVModulus{log2_b, log2_t}, g, cf, as_view(c), key_for);
        els_to(res, out);
        *out_rows = res.count();
    });
}
/// c0 [1, r] CRT basis, c1 [1, r] period basis -> [2, r] CRT basis
int or_bfv_key_switch(void* h, const int64_t* c0, const int64_t* c1, const size_t* base, size_t r, const int64_t* keys,
                      const size_t* digits, size_t d, size_t r_key, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        Base b = base_from(base, r);
        RingEls e0 = els_from(ring, c0, 1, b, Basis::CRTBasis);
        RingEls e1 = els_from(ring, c1, 1, b, Basis::PeriodBasis);
        KeySwitchKey k = key_from(ring, keys, d, digits_from(digits, d), r_key);
        els_to(Bfv(ring, &st).key_switch(as_view(e0), as_view(e1), k), out);
    });
}
/// pb [count, r] period basis (bound <= 2) -> [count, r + ext] CRT basis; crt optional (may be null)
int or_bfv_lift_to_extended(void* h, const int64_t* pb, const int64_t* crt, size_t count, const size_t* base, size_t r,
                            int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        Base b = base_from(base, r);
        RingEls p = els_from(ring, pb, count, b, Basis::PeriodBasis);
        if (crt) {
            RingEls c = els_from(ring, crt, count, b, Basis::CRTBasis);
            RingView cv = as_view(c);
            els_to(Bfv(ring, &st).lift_to_extended(as_view(p), &cv), out);
        } else {
            els_to(Bfv(ring, &st).lift_to_extended(as_view(p), nullptr), out);
        }
    });
}
int or_bfv_rescale_to_base(void* h, const int64_t* x, size_t count, const size_t* base, size_t r, size_t base_len,
                           int64_t t_lo, int64_t t_hi, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        i128 t = (i128)(((u128)(uint64_t)t_hi << 64) | (uint64_t)t_lo);
        RingEls e = els_from(ring, x, count, base_from(base, r), Basis::PeriodBasis);
        els_to(Bfv(ring, &st).rescale_to_base(std::move(e), base_len, t), out);
    });
}
int or_bfv_mod_switch_down(void* h, const int64_t* x, size_t count, const size_t* base, size_t r, size_t new_len,
                           int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        uint64_t st = 0;
        RingEls e = els_from(ring, x, count, base_from(base, r), Basis::PeriodBasis);
        els_to(Bfv(ring, &st).mod_switch_down(as_view(e), new_len), out);
    });
}
/// Wide-accumulator checks (src/ring.rs:2123-2169): rows 1..3 added once, then 0..4, then row 0 `extra` times.
int or_wide_freshness(void* h, const int64_t* data, size_t extra, int64_t* out, int* full_flags) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Base b = ring.initial_rns_base();
        RingEls els = els_from(ring, data, 4, b, Basis::PeriodBasis);
        WideRingEls acc = ring.allocate_wide(4, b);
        acc.add(ring.backend, 1, 3, els.data.view().rows(1, 3), els.bound);
        acc.add(ring.backend, 0, 4, els.data.view(), els.bound);
        for (size_t i = 0; i < extra; i++) acc.add(ring.backend, 0, 1, els.data.view().rows(0, 1), els.bound);
        for (size_t i = 0; i < 4; i++) full_flags[i] = acc.needs_full_reduction(i) ? 1 : 0;
        els_to(ring.reduce_wide(acc, Basis::PeriodBasis), out);
    });
}
/// fma of CRT-basis elements into a fresh wide batch and reduction (ring.fma + reduce_wide)
int or_ring_mul(void* h, const int64_t* a, const int64_t* b, size_t count, const size_t* base, size_t r, int64_t* out) {
    return guarded([&] {
        RingContext& ring = *((BfvHandle*)h)->ring;
        Base bb = base_from(base, r);
        RingEls ea = els_from(ring, a, count, bb, Basis::CRTBasis), eb = els_from(ring, b, count, bb, Basis::CRTBasis);
        WideRingEls acc = ring.allocate_wide(count, bb);
        ring.fma(acc, as_view(ea), as_view(eb));
        els_to(ring.reduce_wide(acc, Basis::CRTBasis), out);
    });
}
}
