// ORACLE — test infrastructure only (see arith.hpp). Restates the ring layer of
// cyclosubfield-dbfv/src/ring.rs on top of the CPU backend restatement:
//   cmod_pow2, cmod, mont_repr, from_mont_repr  src/ring.rs:87-130
//   prime sampling                              src/ring.rs:136-183
//   WideRingEls                                 src/ring.rs:330-532
//   RingContext::new / extension bases          src/ring.rs:622-735
//   allocation, reduce_wide                     src/ring.rs:774-865
//   scalar tensors, mul_scalar, add/sub         src/ring.rs:876-1022
//   q_over_p_inv_tensor, fma*                   src/ring.rs:1029-1090
//   pb_to_crt / crt_to_pb                       src/ring.rs:1094-1161
//   inverse_scalar_tensor, apply_galois         src/ring.rs:1165-1222
//   lprime_element_tensor, transform cache      src/ring.rs:1227-1303
//   CRT kernels                                 src/ring.rs:1320-1415
//   clone_els, element_from_pb_coeffs           src/ring.rs:1424-1461
//   bconv, BConvCache, GadgetBConvCache         src/ring.rs:1517-1852
// Big-integer constants are evaluated modulo each prime (products of primes mod p'), which
// yields the residues feanor-math's big-integer arithmetic produces in the reference.
#pragma once
#include <cmath>
#include <functional>
#include <memory>

#include "cpu_backend.hpp"
#include "field.hpp"

namespace oracle {

enum class Basis { PeriodBasis, CRTBasis };

/// src/ring.rs:87-92
inline i128 cmod_pow2(i128 a, size_t log2_modulus) {
    ORACLE_ASSERT(log2_modulus >= 1 && log2_modulus <= 126, "cmod_pow2 modulus");
    unsigned shift = 128 - (unsigned)log2_modulus;
    i128 result = (i128)((u128)a << shift) >> shift;
    return result == -((i128)1 << (log2_modulus - 1)) ? result + ((i128)1 << log2_modulus) : result;
}
/// src/ring.rs:95-106
inline i128 cmod(i128 a, i128 modulus) {
    i128 modulus_half = modulus / 2;
    i128 result = a % modulus;
    i128 absr = result < 0 ? -result : result;
    if (absr >= modulus_half) {
        if (result < 0) result += modulus;
        else if (result > modulus_half) result -= modulus;
    }
    return result;
}
/// src/ring.rs:109
inline int64_t mont_repr(int64_t x, int64_t p) { return (int64_t)(((i128)x << 64) % (i128)p); }
/// src/ring.rs:111 (truncating)
inline int64_t rmul_mod(int64_t a, int64_t b, int64_t p) { return (int64_t)(((i128)a * b) % p); }
/// src/ring.rs:113-124 (`b.rem_euclid(p)`)
inline int64_t rpow_mod(int64_t b, uint64_t e, int64_t p) {
    int64_t result = 1;
    b = rem_euclid64(b, p);
    while (e > 0) {
        if (e & 1) result = rmul_mod(result, b, p);
        b = rmul_mod(b, b, p);
        e >>= 1;
    }
    return result;
}
/// src/ring.rs:127-130
inline int64_t from_mont_repr(int64_t x, int64_t p) {
    int64_t r_inv = rpow_mod(mont_repr(1, p), (uint64_t)(p - 2), p);
    return rmul_mod(rem_euclid64(x, p), r_inv, p);
}
/// feanor-math `smallest_lift` of a residue in [0, p): the representative in [-(p-1)/2, (p-1)/2].
inline int64_t smallest_lift(int64_t x, int64_t p) {
    x = rem_euclid64(x, p);
    return x > (p - 1) / 2 ? x - p : x;
}
inline int64_t inv_mod_prime(int64_t x, int64_t p) { return rpow_mod(rem_euclid64(x, p), (uint64_t)(p - 2), p); }

/// Deterministic Miller-Rabin for 64-bit integers (the reference calls feanor-math's
/// probabilistic `is_prime(_, _, 10)`, src/ring.rs:139; both agree on every prime it accepts).
inline bool is_prime_u64(uint64_t n) {
    if (n < 2) return false;
    for (uint64_t p : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull}) {
        if (n % p == 0) return n == p;
    }
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) {
        d >>= 1;
        s++;
    }
    auto mulm = [n](uint64_t a, uint64_t b) { return (uint64_t)((u128)a * b % n); };
    auto powm = [&](uint64_t a, uint64_t e) {
        uint64_t r = 1;
        a %= n;
        while (e) {
            if (e & 1) r = mulm(r, a);
            a = mulm(a, a);
            e >>= 1;
        }
        return r;
    };
    for (uint64_t a : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull}) {
        uint64_t x = powm(a, d);
        if (x == 1 || x == n - 1) continue;
        bool composite = true;
        for (int r = 1; r < s; r++) {
            x = mulm(x, x);
            if (x == n - 1) {
                composite = false;
                break;
            }
        }
        if (composite) return false;
    }
    return true;
}

/// src/ring.rs:136-146
inline int64_t largest_prime_leq_congruent_to_one(int64_t leq_than, int64_t m) {
    ORACLE_ASSERT(leq_than > m, "prime search bound");
    int64_t current = leq_than - (leq_than - 1) % m;
    while (!is_prime_u64((uint64_t)current)) {
        current -= m;
        ORACLE_ASSERT(current > 0, "no prime found");
    }
    return current;
}

/// src/ring.rs:150-183
inline std::vector<int64_t> extend_sampled_primes(const std::vector<int64_t>& begin_with, size_t min_bits,
                                                  size_t max_bits, size_t max_bits_each, int64_t m) {
    ORACLE_ASSERT(max_bits > min_bits, "prime bit range");
    std::vector<int64_t> result = begin_with;
    double current_bits = 0;
    for (int64_t p : result) current_bits += std::log2((double)p);
    ORACLE_ASSERT((size_t)std::floor(current_bits) < max_bits, "prime bit range");
    int64_t current_upper_bound = (int64_t)1 << max_bits_each;
    while (current_bits < (double)min_bits) {
        double remaining = (double)min_bits - current_bits;
        double allowed;
        if (remaining < (double)max_bits_each) {
            allowed = std::fmin((double)max_bits - current_bits, (double)max_bits_each);
        } else {
            double required = std::ceil(remaining / (double)max_bits_each);
            allowed = std::fmin(((double)max_bits - current_bits) / required, (double)max_bits_each);
        }
        current_upper_bound = std::min(current_upper_bound, (int64_t)1 << (size_t)std::floor(allowed));
        int64_t prime = largest_prime_leq_congruent_to_one(current_upper_bound, m);
        current_upper_bound = prime - 1;
        while (std::find(begin_with.begin(), begin_with.end(), prime) != begin_with.end()) {
            prime = largest_prime_leq_congruent_to_one(current_upper_bound, m);
            current_upper_bound = prime - 1;
        }
        current_bits += std::log2((double)prime);
        result.push_back(prime);
    }
    return result;
}

/// Bit length of a product of primes (= ceil(log2) for a non-power-of-two), computed exactly.
inline size_t product_bitlen(const std::vector<int64_t>& primes) {
    std::vector<uint32_t> limbs{1};
    for (int64_t p : primes) {
        uint64_t lo = (uint64_t)p & 0xffffffffu, hi = (uint64_t)p >> 32;
        std::vector<uint32_t> out(limbs.size() + 3, 0);
        for (size_t i = 0; i < limbs.size(); i++) {
            for (int part = 0; part < 2; part++) {
                u128 carry = 0;
                uint64_t f = part == 0 ? lo : hi;
                size_t k = i + part;
                u128 prod = (u128)limbs[i] * f;
                while (prod != 0 || carry != 0) {
                    u128 s = (u128)out[k] + (uint32_t)prod + carry;
                    out[k] = (uint32_t)s;
                    carry = s >> 32;
                    prod >>= 32;
                    k++;
                }
            }
        }
        while (out.size() > 1 && out.back() == 0) out.pop_back();
        limbs = out;
    }
    size_t top = limbs.size() - 1;
    size_t bits = 32 * top;
    uint32_t v = limbs[top];
    while (v) {
        bits++;
        v >>= 1;
    }
    return bits;
}

typedef std::vector<size_t> Base;
typedef std::vector<MontgomeryModulus> Mods;
typedef std::vector<const CpuNTTPlan*> Plans;

/// A batch of ring elements (src/ring.rs:198-208).
struct RingEls {
    Base rns_base;
    Basis basis;
    u128 bound;
    Tensor<int64_t> data;
    size_t count() const { return data.shape[0]; }
};

/// A (mutable) view of a batch (src/ring.rs:211-235).
struct RingView {
    Base rns_base;
    Basis basis;
    u128 bound;
    V64 data;
    size_t count() const { return data.shape[0]; }
    RingView rows(size_t s, size_t e) const { return RingView{rns_base, basis, bound, data.rows(s, e)}; }
    RingView restrict_base(size_t len) const {
        ORACLE_ASSERT(len <= rns_base.size(), "restrict_base");
        return RingView{Base(rns_base.begin(), rns_base.begin() + len), basis, bound, data.base_range(0, len)};
    }
};
inline RingView as_view(const RingEls& e) { return RingView{e.rns_base, e.basis, e.bound, e.data.view()}; }

/// src/ring.rs:330-532
struct WideRingEls {
    Base rns_base;
    Tensor<i128> data;
    Tensor<int64_t> one, neg_one;
    int64_t max_p, min_p;
    std::vector<u128> bound;

    size_t count() const { return bound.size(); }
    void record_step(size_t rs, size_t re, u128 step) {
        for (size_t i = rs; i < re; i++) {
            u128 b = bound[i] + step;
            ORACLE_ASSERT(b >= bound[i] && b <= (u128)I128_MAX, "wide ring element overflow");
            bound[i] = b;
        }
    }
    bool needs_full_reduction(size_t row) const { return bound[row] > ((u128)min_p << 63); }

    /// src/ring.rs:373-413
    void accumulate(const CpuBackend& be, size_t rs, size_t re, V64 lhs, V64 rhs) {
        auto slice_operand = [&](V64 t, size_t s, size_t e) { return t.shape[0] == 1 ? t : t.rows(s - rs, e - rs); };
        size_t start = rs;
        while (start < re) {
            bool fresh = bound[start] == 0;
            size_t end = start + 1;
            while (end < re && (bound[end] == 0) == fresh) end++;
            V128 dst = data.view().rows(start, end);
            if (fresh) be.hal_mul_i64(dst, slice_operand(lhs, start, end), slice_operand(rhs, start, end));
            else be.hal_fma_i64(dst, slice_operand(lhs, start, end), slice_operand(rhs, start, end));
            start = end;
        }
    }
    u128 maxp2() const { return (u128)max_p * (u128)max_p; }
    /// src/ring.rs:421-436
    void fma(const CpuBackend& be, size_t rs, size_t re, V64 lhs, u128 lb, V64 rhs, u128 rb) {
        accumulate(be, rs, re, lhs, rhs);
        record_step(rs, re, lb * rb * maxp2());
    }
    void fma_all(const CpuBackend& be, V64 lhs, u128 lb, V64 rhs, u128 rb) { fma(be, 0, count(), lhs, lb, rhs, rb); }
    /// src/ring.rs:460-485
    void inner_product(const CpuBackend& be, size_t rs, size_t re,
                       const std::vector<std::tuple<V64, u128, V64, u128>>& terms) {
        ORACLE_ASSERT(!terms.empty(), "inner product needs at least one term");
        for (size_t i = rs; i < re; i++) ORACLE_ASSERT(bound[i] == 0, "inner_product requires fresh rows");
        std::vector<V64> l, r;
        u128 step = 0;
        for (auto& t : terms) {
            l.push_back(std::get<0>(t));
            r.push_back(std::get<2>(t));
            step += std::get<1>(t) * std::get<3>(t) * maxp2();
        }
        be.hal_inner_product_i64(data.view().rows(rs, re), l, r);
        record_step(rs, re, step);
    }
    /// src/ring.rs:490-493
    void fma_unbounded(const CpuBackend& be, size_t rs, size_t re, V64 lhs, V64 rhs) {
        accumulate(be, rs, re, lhs, rhs);
        record_step(rs, re, (u128)max_p << 63);
    }
    /// src/ring.rs:503-531
    void add(const CpuBackend& be, size_t rs, size_t re, V64 src, u128 sb) {
        accumulate(be, rs, re, src, one.view());
        record_step(rs, re, sb * maxp2());
    }
    void sub(const CpuBackend& be, size_t rs, size_t re, V64 src, u128 sb) {
        accumulate(be, rs, re, src, neg_one.view());
        record_step(rs, re, sb * maxp2());
    }
};

struct RnsFactor {
    int64_t p;
    MontgomeryModulus modulus;
    bool supports_transform;
};

/// src/ring.rs:558-567
struct RnsFactorKernels {
    std::vector<int64_t> crt_kernel_lprime, crt_kernel_k, inv_crt_kernel_lprime, inv_crt_kernel_k;
};

/// src/ring.rs:581-592
struct TransformCache {
    Base rns_base;
    Mods mods;
    std::vector<CpuNTTPlan> ntts_lprime, ntts_k;
    Tensor<int64_t> crt_kernel_lprime, crt_kernel_k, inv_crt_kernel_lprime, inv_crt_kernel_k;
    Plans plans_lprime() const {
        Plans r;
        for (auto& p : ntts_lprime) r.push_back(&p);
        return r;
    }
    Plans plans_k() const {
        Plans r;
        for (auto& p : ntts_k) r.push_back(&p);
        return r;
    }
};

struct RingContext;

/// src/ring.rs:1595-1702
struct BConvCache {
    Base src_rns_base, dst_rns_base;
    size_t log2_qtilde;
    Tensor<int64_t> q_over_p_inv, matrix, q_mod_p_;
    size_t acc_before_reduce;
};

/// src/ring.rs:1714-1852
struct GadgetBConvCache {
    Base rns_base;
    std::vector<std::pair<size_t, size_t>> digits;
    size_t log2_qtilde;
    Tensor<int64_t> d_over_p_inv, matrix, d_mod_p;
    size_t acc_before_reduce;
};

/// A big-integer scalar, given by its residue modulo any prime (in [0, p)).
typedef std::function<int64_t(int64_t)> BigResidue;

struct RingContext {
    CpuBackend backend;
    FieldDescriptor field;
    std::vector<RnsFactor> rns_factors;
    size_t initial_rns_base_len;
    size_t t_bits;
    size_t sparse_key_encaps_len;
    std::vector<std::unique_ptr<TransformCache>> transform_cache;
    std::map<int64_t, std::shared_ptr<RnsFactorKernels>> rns_factor_kernels;
    std::vector<std::unique_ptr<BConvCache>> bconv_cache;
    std::vector<std::unique_ptr<GadgetBConvCache>> gadget_bconv_cache;
    std::map<std::vector<int64_t>, std::pair<CpuPermutationPlan, CpuPermutationPlan>> permutation_cache;

    static constexpr size_t EXTENDED_Q_EXTRA_BITS = 60;  // src/ring.rs:82

    /// src/ring.rs:622-652
    static std::unique_ptr<RingContext> create(const FieldDescriptor& field, size_t log2_q_lo, size_t log2_q_hi,
                                               size_t t_bits) {
        auto r = std::make_unique<RingContext>();
        r->field = field;
        int64_t rou = (int64_t)field.rou_order();
        std::vector<int64_t> base = extend_sampled_primes({}, log2_q_lo, log2_q_hi, 57, rou);
        std::vector<int64_t> ext =
            extend_sampled_primes(base, 2 * log2_q_hi + EXTENDED_Q_EXTRA_BITS + t_bits,
                                  2 * log2_q_hi + EXTENDED_Q_EXTRA_BITS + t_bits + 30, 57, rou);
        r->initial_rns_base_len = base.size();
        r->t_bits = t_bits;
        r->sparse_key_encaps_len = std::min<size_t>(3, base.size());
        for (int64_t p : ext) r->add_rns_factor(p, true);
        return r;
    }
    /// src/ring.rs:657-677 (test-only constructor without transform support)
    static std::unique_ptr<RingContext> create_raw(const FieldDescriptor& field, const std::vector<int64_t>& primes) {
        auto r = std::make_unique<RingContext>();
        r->field = field;
        r->initial_rns_base_len = primes.size();
        r->t_bits = 0;
        r->sparse_key_encaps_len = std::min<size_t>(3, primes.size());
        for (int64_t p : primes) r->add_rns_factor(p, false);
        return r;
    }
    void add_rns_factor(int64_t p, bool transform) {
        ORACLE_ASSERT(p >= ((int64_t)1 << 40) && p <= ((int64_t)1 << 57) - 1, "RNS factor size");
        for (auto& f : rns_factors) ORACLE_ASSERT(f.p != p, "duplicate RNS factor");
        if (transform) ORACLE_ASSERT((p - 1) % (int64_t)field.rou_order() == 0, "RNS factor incompatible with the field");
        rns_factors.push_back(RnsFactor{p, backend.hal_create_modulus(p), transform});
    }

    size_t n() const { return field.deg_l; }
    Base initial_rns_base() const {
        Base b;
        for (size_t i = 0; i < initial_rns_base_len; i++) b.push_back(i);
        return b;
    }
    Base sparse_key_encaps_rns_base() const {
        Base b;
        for (size_t i = 0; i < sparse_key_encaps_len; i++) b.push_back(i);
        return b;
    }
    int64_t prime(size_t idx) const { return rns_factors[idx].p; }
    std::vector<int64_t> primes_of(const Base& base) const {
        std::vector<int64_t> r;
        for (size_t i : base) r.push_back(rns_factors[i].p);
        return r;
    }
    /// Q(base) mod p (src/ring.rs:748-750, evaluated modulo p).
    int64_t modulus_mod(const Base& base, int64_t p) const {
        int64_t r = 1 % p;
        for (size_t i : base) r = rmul_mod(r, rns_factors[i].p % p, p);
        return r;
    }
    double log2_modulus_of(const Base& base) const {
        double s = 0;
        for (size_t i : base) s += std::log2((double)rns_factors[i].p);
        return s;
    }
    /// src/ring.rs:716-731
    Base extension_rns_base_for(const Base& base) const {
        for (size_t i : base) ORACLE_ASSERT(i < initial_rns_base_len, "extension of non-initial base");
        double required = (double)(product_bitlen(primes_of(base)) + t_bits + EXTENDED_Q_EXTRA_BITS);
        Base result;
        double bits = 0;
        for (size_t idx = initial_rns_base_len; idx < rns_factors.size(); idx++) {
            if (bits >= required) break;
            result.push_back(idx);
            bits += std::log2((double)rns_factors[idx].p);
        }
        ORACLE_ASSERT(bits >= required, "extension pool too small for lifted multiplication over this base");
        return result;
    }
    Mods mods_for(const Base& base) const {
        Mods m;
        for (size_t i : base) m.push_back(rns_factors[i].modulus);
        return m;
    }
    int64_t max_p_of(const Base& base) const {
        int64_t m = 1;
        for (size_t i : base) m = std::max(m, rns_factors[i].p);
        return m;
    }
    int64_t min_p_of(const Base& base) const {
        int64_t m = INT64_MAX;
        for (size_t i : base) m = std::min(m, rns_factors[i].p);
        return base.empty() ? 1 : m;
    }

    // ---- allocation (src/ring.rs:774-809) ----
    RingEls allocate_in_basis(size_t count, const Base& base, Basis basis) const {
        return RingEls{base, basis, 1, Tensor<int64_t>(Shape{count, base.size(), field.deg_lprime, field.deg_k})};
    }
    RingEls allocate(size_t count, const Base& base) const { return allocate_in_basis(count, base, Basis::PeriodBasis); }
    WideRingEls allocate_wide(size_t count, const Base& base) const {
        WideRingEls w;
        w.rns_base = base;
        w.data = Tensor<i128>(Shape{count, base.size(), field.deg_lprime, field.deg_k});
        w.one = scalar_tensor(base, 1);
        w.neg_one = scalar_tensor(base, -1);
        w.max_p = max_p_of(base);
        w.min_p = min_p_of(base);
        w.bound.assign(count, 0);
        return w;
    }

    // ---- reduce_wide (src/ring.rs:814-865) ----
    RingEls reduce_wide(const WideRingEls& wide, Basis basis) const { return reduce_wide_rows(wide, 0, wide.count(), basis); }
    RingEls reduce_wide_rows(const WideRingEls& wide, size_t rs, size_t re, Basis basis) const {
        RingEls result = allocate_in_basis(re - rs, wide.rns_base, basis);
        reduce_wide_tensor(result.data.view(), wide, rs, re);
        return result;
    }
    void reduce_wide_into(RingView dst, const WideRingEls& wide) const {
        ORACLE_ASSERT(dst.rns_base == wide.rns_base, "reduce_wide_into base");
        reduce_wide_tensor(dst.data, wide, 0, wide.count());
    }
    void reduce_wide_tensor(V64 dst, const WideRingEls& wide, size_t rs, size_t re) const {
        Mods mods = mods_for(wide.rns_base);
        size_t start = rs;
        while (start < re) {
            bool full = wide.needs_full_reduction(start);
            size_t end = start + 1;
            while (end < re && wide.needs_full_reduction(end) == full) end++;
            V64 dst_run = dst.rows(start - rs, end - rs);
            V128 wide_run = wide.data.view().rows(start, end);
            if (full) {
                backend.hal_red_mont64_double(dst_run, wide_run, mods);
                backend.hal_i64_to_mont64(dst_run, mods);
            } else {
                backend.hal_red_mont64(dst_run, wide_run, mods);
            }
            start = end;
        }
    }

    // ---- scalar tensors (src/ring.rs:876-920, 1029-1043, 1165-1177) ----
    Tensor<int64_t> import_tensor(const std::vector<int64_t>& values, Shape shape) const {
        Tensor<int64_t> t = backend.hal_allocate_i64(shape);
        backend.hal_import(t.view(), values.data(), values.size());
        return t;
    }
    Tensor<int64_t> scalar_tensor(const Base& base, i128 scalar) const {
        std::vector<int64_t> v;
        for (size_t i : base) {
            int64_t p = rns_factors[i].p;
            v.push_back(mont_repr((int64_t)(scalar % (i128)p), p));
        }
        return import_tensor(v, Shape{1, base.size(), 1, 1});
    }
    Tensor<int64_t> scalar_tensor_big(const Base& base, const BigResidue& scalar) const {
        std::vector<int64_t> v;
        for (size_t i : base) {
            int64_t p = rns_factors[i].p;
            v.push_back(mont_repr(smallest_lift(scalar(p), p), p));
        }
        return import_tensor(v, Shape{1, base.size(), 1, 1});
    }
    Tensor<int64_t> inverse_scalar_tensor(const Base& base, const BigResidue& scalar) const {
        std::vector<int64_t> v;
        for (size_t i : base) {
            int64_t p = rns_factors[i].p;
            int64_t s = rem_euclid64(scalar(p), p);
            ORACLE_ASSERT(s != 0, "scalar not invertible");
            v.push_back(mont_repr(smallest_lift(inv_mod_prime(s, p), p), p));
        }
        return import_tensor(v, Shape{1, base.size(), 1, 1});
    }
    Tensor<int64_t> q_over_p_inv_tensor(const Base& base, i128 scale) const {
        std::vector<int64_t> v;
        for (size_t k = 0; k < base.size(); k++) {
            int64_t p = rns_factors[base[k]].p;
            int64_t q_over_p = 1;
            for (size_t l = 0; l < base.size(); l++)
                if (l != k) q_over_p = rmul_mod(q_over_p, rns_factors[base[l]].p % p, p);
            int64_t s = (int64_t)rem_euclid128(scale, (i128)p);
            v.push_back(smallest_lift(rmul_mod(inv_mod_prime(q_over_p, p), s, p), p));
        }
        return import_tensor(v, Shape{1, base.size(), 1, 1});
    }
    void assert_mul_mont_safe(u128 bound, const Base& base) const {
        u128 prod = bound * (u128)max_p_of(base);
        ORACLE_ASSERT(bound == 0 || (prod / bound == (u128)max_p_of(base) && prod <= ((u128)1 << 63)),
                      "representatives too large for a montgomery multiplication");
    }
    void mul_scalar(RingEls& els, i128 scalar) const {
        assert_mul_mont_safe(els.bound, els.rns_base);
        Tensor<int64_t> t = scalar_tensor(els.rns_base, scalar);
        backend.hal_mul_mont64(els.data.view(), t.view(), mods_for(els.rns_base));
        els.bound = 1;
    }
    void mul_scalar_big(RingEls& els, const BigResidue& scalar) const {
        assert_mul_mont_safe(els.bound, els.rns_base);
        Tensor<int64_t> t = scalar_tensor_big(els.rns_base, scalar);
        backend.hal_mul_mont64(els.data.view(), t.view(), mods_for(els.rns_base));
        els.bound = 1;
    }

    // ---- wide accumulation helpers (src/ring.rs:965-1090) ----
    void add(WideRingEls& wide, const RingView& src) const {
        ORACLE_ASSERT(wide.rns_base == src.rns_base, "add base");
        wide.add(backend, 0, wide.count(), src.data, src.bound);
    }
    void sub(WideRingEls& wide, const RingView& src) const {
        ORACLE_ASSERT(wide.rns_base == src.rns_base, "sub base");
        wide.sub(backend, 0, wide.count(), src.data, src.bound);
    }
    void add_sub_els(RingEls& dst, const RingView& src, bool subtract) const {
        ORACLE_ASSERT(dst.rns_base == src.rns_base && dst.basis == src.basis, "add_els operands");
        u128 new_bound = dst.bound + src.bound;
        ORACLE_ASSERT(new_bound * (u128)max_p_of(dst.rns_base) <= I64_MAX_U, "unreduced addition could overflow");
        if (subtract) backend.hal_sub_i64(dst.data.view(), src.data);
        else backend.hal_add_i64(dst.data.view(), src.data);
        dst.bound = new_bound;
    }
    void add_els(RingEls& dst, const RingView& src) const { add_sub_els(dst, src, false); }
    void sub_els(RingEls& dst, const RingView& src) const { add_sub_els(dst, src, true); }
    void fma(WideRingEls& wide, const RingView& lhs, const RingView& rhs) const {
        ORACLE_ASSERT(lhs.rns_base == rhs.rns_base && wide.rns_base == lhs.rns_base, "fma bases");
        ORACLE_ASSERT(lhs.basis == Basis::CRTBasis && rhs.basis == Basis::CRTBasis, "fma requires CRT basis");
        wide.fma_all(backend, lhs.data, lhs.bound, rhs.data, rhs.bound);
    }
    void fma_scalar(WideRingEls& wide, const RingView& els, i128 scalar) const {
        Tensor<int64_t> t = scalar_tensor(els.rns_base, scalar);
        wide.fma_all(backend, els.data, els.bound, t.view(), 1);
    }
    void fma_scalar_big(WideRingEls& wide, const RingView& els, const BigResidue& scalar) const {
        Tensor<int64_t> t = scalar_tensor_big(els.rns_base, scalar);
        wide.fma_all(backend, els.data, els.bound, t.view(), 1);
    }

    // ---- CRT transforms (src/ring.rs:1094-1161) ----
    void pb_to_crt(RingEls& els) {
        ORACLE_ASSERT(els.basis == Basis::PeriodBasis, "pb_to_crt basis");
        ORACLE_ASSERT(els.bound <= 2, "basis transforms require representatives bounded by 2p");
        pb_to_crt_tensor(els.data.view(), els.rns_base);
        els.basis = Basis::CRTBasis;
        els.bound = 1;
    }
    void crt_to_pb(RingEls& els) {
        ORACLE_ASSERT(els.basis == Basis::CRTBasis, "crt_to_pb basis");
        ORACLE_ASSERT(els.bound <= 2, "basis transforms require representatives bounded by 2p");
        crt_to_pb_tensor(els.data.view(), els.rns_base);
        els.basis = Basis::PeriodBasis;
        els.bound = 1;
    }
    void pb_to_crt_tensor(V64 data, const Base& base) {
        TransformCache& c = transform_cache_for(base);
        backend.hal_ntt_mul_mont64_dim(data, c.plans_lprime(), DataDim::Dim2, c.crt_kernel_lprime.view(), c.mods);
        backend.hal_ntt_mul_mont64_dim(data, c.plans_k(), DataDim::Dim3, c.crt_kernel_k.view(), c.mods);
        backend.hal_intt_mont64(data, c.plans_lprime(), c.plans_k());
    }
    void crt_to_pb_tensor(V64 data, const Base& base) {
        TransformCache& c = transform_cache_for(base);
        backend.hal_ntt_mul_mont64_dim(data, c.plans_lprime(), DataDim::Dim2, c.inv_crt_kernel_lprime.view(), c.mods);
        backend.hal_ntt_mul_mont64_dim(data, c.plans_k(), DataDim::Dim3, c.inv_crt_kernel_k.view(), c.mods);
        backend.hal_intt_mont64(data, c.plans_lprime(), c.plans_k());
    }

    // ---- Galois automorphisms (src/ring.rs:1183-1222) ----
    std::pair<CpuPermutationPlan, CpuPermutationPlan>& galois_perms(uint64_t g) {
        std::vector<int64_t> shift = field.gal_to_shift(g);
        auto it = permutation_cache.find(shift);
        if (it != permutation_cache.end()) return it->second;
        size_t lf = field.lprime_factor_count;
        std::vector<size_t> orders = field.lq_cyclic_orders();
        std::vector<size_t> o1(orders.begin(), orders.begin() + lf), o2(orders.begin() + lf, orders.end());
        std::vector<size_t> s1, s2;
        for (size_t i = 0; i < shift.size(); i++) (i < lf ? s1 : s2).push_back((size_t)shift[i]);
        auto plans = std::make_pair(backend.hal_create_permutation(o1, s1), backend.hal_create_permutation(o2, s2));
        return permutation_cache.emplace(shift, plans).first->second;
    }
    void apply_galois(RingEls& dst, const RingView& src, uint64_t g) {
        ORACLE_ASSERT(dst.rns_base == src.rns_base, "apply_galois base");
        dst.basis = src.basis;
        dst.bound = src.bound;
        auto& perms = galois_perms(g);
        Tensor<int64_t> tmp = backend.hal_allocate_i64(src.data.shape);
        backend.hal_permute(tmp.view(), src.data, perms.first, DataDim::Dim2);
        backend.hal_permute(dst.data.view(), tmp.view(), perms.second, DataDim::Dim3);
    }

    /// src/ring.rs:1227-1250
    Tensor<int64_t> lprime_element_tensor(const Base& base, const std::vector<i128>& coeffs) {
        ORACLE_ASSERT(coeffs.size() == field.deg_lprime, "lprime element length");
        std::vector<int64_t> values;
        for (size_t idx : base) {
            int64_t p = rns_factors[idx].p;
            for (i128 c : coeffs) values.push_back(mont_repr((int64_t)(c % (i128)p), p));
        }
        Tensor<int64_t> result = import_tensor(values, Shape{1, base.size(), field.deg_lprime, 1});
        TransformCache& c = transform_cache_for(base);
        backend.hal_ntt_mul_mont64_dim(result.view(), c.plans_lprime(), DataDim::Dim2, c.crt_kernel_lprime.view(),
                                       c.mods);
        backend.hal_intt_mont64_dim(result.view(), c.plans_lprime(), DataDim::Dim2);
        return result;
    }

    // ---- transform cache (src/ring.rs:1252-1303, 1320-1415) ----
    TransformCache& transform_cache_for(const Base& base) {
        for (auto& c : transform_cache)
            if (c->rns_base == base) return *c;
        auto c = std::make_unique<TransformCache>();
        c->rns_base = base;
        c->mods = mods_for(base);
        size_t r = base.size(), dl = field.deg_lprime, dk = field.deg_k;
        std::vector<int64_t> kl, kk, ikl, ikk;
        for (size_t idx : base) {
            ORACLE_ASSERT(rns_factors[idx].supports_transform, "RNS factor doesn't support the basis transforms");
            int64_t p = rns_factors[idx].p;
            c->ntts_lprime.push_back(backend.hal_create_ntt_plan(rns_factors[idx].modulus, field.lprime_orders()));
            c->ntts_k.push_back(backend.hal_create_ntt_plan(rns_factors[idx].modulus, field.k_orders()));
            std::shared_ptr<RnsFactorKernels> kern = kernels_for(p, c->ntts_lprime.back(), c->ntts_k.back());
            kl.insert(kl.end(), kern->crt_kernel_lprime.begin(), kern->crt_kernel_lprime.end());
            kk.insert(kk.end(), kern->crt_kernel_k.begin(), kern->crt_kernel_k.end());
            ikl.insert(ikl.end(), kern->inv_crt_kernel_lprime.begin(), kern->inv_crt_kernel_lprime.end());
            ikk.insert(ikk.end(), kern->inv_crt_kernel_k.begin(), kern->inv_crt_kernel_k.end());
        }
        c->crt_kernel_lprime = import_tensor(kl, Shape{1, r, dl, 1});
        c->crt_kernel_k = import_tensor(kk, Shape{1, r, 1, dk});
        c->inv_crt_kernel_lprime = import_tensor(ikl, Shape{1, r, dl, 1});
        c->inv_crt_kernel_k = import_tensor(ikk, Shape{1, r, 1, dk});
        transform_cache.push_back(std::move(c));
        return *transform_cache.back();
    }
    std::shared_ptr<RnsFactorKernels> kernels_for(int64_t p, const CpuNTTPlan& ntt_lprime, const CpuNTTPlan& ntt_k) {
        auto it = rns_factor_kernels.find(p);
        if (it != rns_factor_kernels.end()) return it->second;
        auto k = std::make_shared<RnsFactorKernels>(compute_rns_factor_kernels(p, ntt_lprime, ntt_k));
        rns_factor_kernels[p] = k;
        return k;
    }
    /// src/ring.rs:1338-1415
    RnsFactorKernels compute_rns_factor_kernels(int64_t p, const CpuNTTPlan& ntt_lprime, const CpuNTTPlan& ntt_k) {
        int64_t m = (int64_t)field.m;
        int64_t zeta = 0;
        for (int64_t candidate = 2;; candidate++) {
            zeta = rpow_mod(candidate, (uint64_t)((p - 1) / m), p);
            bool ok = true;
            for (uint64_t f : field.m_factors)
                if (rpow_mod(zeta, (uint64_t)(m / (int64_t)f), p) == 1) ok = false;
            if (ok) break;
        }
        int64_t zeta_mprime = rpow_mod(zeta, crt2(1, field.m_prime, 0, field.m_k()), p);
        int64_t zeta_mk = rpow_mod(zeta, crt2(0, field.m_prime, 1, field.m_k()), p);
        auto compute_kernel = [&](int64_t zeta_part, uint64_t part_order, const std::vector<uint64_t>& subgroup,
                                  const std::vector<uint64_t>& transversal) {
            std::vector<int64_t> powers;
            int64_t current = 1;
            for (uint64_t i = 0; i < part_order; i++) {
                powers.push_back(current);
                current = rmul_mod(current, zeta_part, p);
            }
            std::vector<int64_t> out;
            for (uint64_t g : transversal) {
                uint64_t g_inv = inv_mod(g, field.m);
                int64_t sum = 0;
                for (uint64_t x : subgroup) {
                    uint64_t exponent = (uint64_t)(((u128)x * g_inv) % field.m) % part_order;
                    sum = (sum + powers[exponent]) % p;
                }
                out.push_back(sum);
            }
            return out;
        };
        std::vector<int64_t> kernel_lprime =
            compute_kernel(zeta_mprime, field.m_prime, field.gal_mprime_lprime, field.lprime_q_transversal());
        std::vector<int64_t> kernel_k = compute_kernel(zeta_mk, field.m_k(), field.gal_mk_k, field.kq_transversal());
        auto to_ntt_domain = [&](const std::vector<int64_t>& kernel, const CpuNTTPlan& plan, Shape shape,
                                 DataDim dim) {
            std::vector<int64_t> mk;
            for (int64_t x : kernel) mk.push_back(mont_repr(x, p));
            Tensor<int64_t> t = import_tensor(mk, shape);
            backend.hal_ntt_mont64_dim(t.view(), Plans{&plan}, dim);
            std::vector<int64_t> result(kernel.size());
            backend.hal_export(t.view(), result.data(), result.size());
            for (auto& x : result) x = rem_euclid64(x, p);
            return result;
        };
        size_t dl = field.deg_lprime, dk = field.deg_k;
        RnsFactorKernels k;
        k.crt_kernel_lprime = to_ntt_domain(kernel_lprime, ntt_lprime, Shape{1, 1, dl, 1}, DataDim::Dim2);
        k.crt_kernel_k = to_ntt_domain(kernel_k, ntt_k, Shape{1, 1, 1, dk}, DataDim::Dim3);
        auto invert = [&](const std::vector<int64_t>& kernel) {
            std::vector<int64_t> out;
            for (int64_t x : kernel) {
                int64_t plain = from_mont_repr(x, p);
                ORACLE_ASSERT(plain != 0, "CRT kernel is not invertible");
                out.push_back(mont_repr(rpow_mod(plain, (uint64_t)(p - 2), p), p));
            }
            return out;
        };
        k.inv_crt_kernel_lprime = invert(k.crt_kernel_lprime);
        k.inv_crt_kernel_k = invert(k.crt_kernel_k);
        return k;
    }

    // ---- copies (src/ring.rs:1418-1461) ----
    RingEls clone_els(const RingView& els) const {
        RingEls result = allocate_in_basis(els.count(), els.rns_base, els.basis);
        backend.hal_assign(result.data.view(), els.data);
        result.bound = els.bound;
        return result;
    }
    RingEls element_from_pb_coeffs(const Base& base, const std::vector<i128>& coeffs) const {
        ORACLE_ASSERT(coeffs.size() == n(), "element length");
        std::vector<int64_t> values;
        for (size_t idx : base) {
            int64_t p = rns_factors[idx].p;
            for (i128 c : coeffs) values.push_back(mont_repr((int64_t)(c % (i128)p), p));
        }
        RingEls result = allocate(1, base);
        backend.hal_import(result.data.view(), values.data(), values.size());
        return result;
    }

    // ---- base conversion (src/ring.rs:1517-1702) ----
    void bconv(RingEls& dst, RingEls& src) {
        assert_mul_mont_safe(src.bound, src.rns_base);
        dst.basis = src.basis;
        dst.bound = 1;
        bconv_tensors(dst.data.view(), dst.rns_base, src.data.view(), src.rns_base);
    }
    BConvCache& bconv_cache_for(const Base& src_base, const Base& dst_base) {
        for (auto& c : bconv_cache)
            if (c->src_rns_base == src_base && c->dst_rns_base == dst_base) return *c;
        bconv_cache.push_back(std::make_unique<BConvCache>(make_bconv_cache(src_base, dst_base)));
        return *bconv_cache.back();
    }
    /// src/ring.rs:1606-1661
    BConvCache make_bconv_cache(const Base& src_base, const Base& dst_base) {
        size_t r = src_base.size(), r_ = dst_base.size();
        int64_t max_p = 0, min_p = INT64_MAX;
        for (size_t i : src_base) max_p = std::max(max_p, rns_factors[i].p), min_p = std::min(min_p, rns_factors[i].p);
        for (size_t i : dst_base) max_p = std::max(max_p, rns_factors[i].p);
        BConvCache c;
        c.src_rns_base = src_base;
        c.dst_rns_base = dst_base;
        size_t l2 = 0;
        for (u128 v = (u128)(4 * (i128)r * max_p + 1); v; v >>= 1) l2++;
        c.log2_qtilde = std::max<size_t>(64, l2);
        ORACLE_ASSERT(c.log2_qtilde <= 126, "log2 qtilde");
        i128 qtilde = (i128)1 << c.log2_qtilde;
        i128 cvmax = (qtilde - 1) / min_p + 1;
        ORACLE_ASSERT(cvmax <= INT64_MAX, "coefficients of correction vector don't fit into an i64");
        c.acc_before_reduce = (size_t)(I128_MAX / ((i128)max_p * max_p));
        ORACLE_ASSERT(c.acc_before_reduce >= 16, "acc_before_reduce");
        c.q_over_p_inv = q_over_p_inv_tensor(src_base, 1);
        std::vector<int64_t> mat;
        for (size_t i = 0; i < r_; i++) {
            int64_t pp = rns_factors[dst_base[i]].p;
            int64_t r_sqr = rmul_mod(mont_repr(1, pp), mont_repr(1, pp), pp);
            for (size_t j = 0; j < r; j++) {
                int64_t value = 1;
                for (size_t l = 0; l < r; l++)
                    if (l != j) value = rmul_mod(value, rns_factors[src_base[l]].p % pp, pp);
                mat.push_back(smallest_lift(rmul_mod(rem_euclid64(value, pp), rem_euclid64(r_sqr, pp), pp), pp));
            }
        }
        for (size_t j = 0; j < r; j++) mat.push_back((int64_t)rounded_div(qtilde, (i128)rns_factors[src_base[j]].p));
        c.matrix = import_tensor(mat, Shape{1, r_ + 1, r, 1});
        std::vector<int64_t> qm;
        for (size_t i = 0; i < r_; i++) {
            int64_t pp = rns_factors[dst_base[i]].p;
            int64_t q_mod = rem_euclid64(modulus_mod(src_base, pp), pp);
            int64_t neg_r = rem_euclid64(-mont_repr(1, pp), pp);
            qm.push_back(smallest_lift(rmul_mod(q_mod, neg_r, pp), pp));
        }
        c.q_mod_p_ = import_tensor(qm, Shape{1, r_, 1, 1});
        return c;
    }
    /// src/ring.rs:1663-1701
    void bconv_tensors(V64 dst, const Base& dst_base, V64 src, const Base& src_base) {
        BConvCache& c = bconv_cache_for(src_base, dst_base);
        size_t r = src_base.size(), r_ = dst_base.size();
        Shape shape{src.shape[0], 1, src.shape[2], src.shape[3]};
        ORACLE_ASSERT(dst.shape == (Shape{shape[0], r_, shape[2], shape[3]}), "bconv dst shape");
        Mods src_mods = mods_for(src_base), dst_mods = mods_for(dst_base);
        backend.hal_mul_mont64(src, c.q_over_p_inv.view(), src_mods);
        Tensor<i128> correction = backend.hal_allocate_i128(shape);
        Tensor<i128> tmp = backend.hal_allocate_i128(Shape{shape[0], r_ + 1, shape[2], shape[3]});
        for (size_t j = 0, chunk = 0; j < r; j += c.acc_before_reduce, chunk++) {
            size_t e = std::min(j + c.acc_before_reduce, r);
            backend.hal_matmul_i64(tmp.view(), c.matrix.view().slice(0, 1, 0, r_ + 1, j, e, 0, 1),
                                   src.slice(0, src.shape[0], j, e, 0, src.shape[2], 0, src.shape[3]));
            V128 vals = tmp.view().base_range(0, r_), corr = tmp.view().base_range(r_, r_ + 1);
            if (chunk == 0) {
                backend.hal_red_mont64_double(dst, vals, dst_mods);
                backend.hal_assign_i128(correction.view(), corr);
            } else {
                backend.hal_add_red_mont64_double(dst, vals, dst_mods);
                backend.hal_add_i128(correction.view(), corr);
            }
        }
        backend.hal_bconv_correct_mont64(dst, correction.view(), c.q_mod_p_.view(), dst_mods, c.log2_qtilde);
        backend.hal_i64_to_mont64(dst, dst_mods);
    }

    // ---- gadget base conversion (src/ring.rs:1537-1574, 1714-1852) ----
    GadgetBConvCache& gadget_cache_for(const Base& base, const std::vector<std::pair<size_t, size_t>>& digits) {
        for (auto& c : gadget_bconv_cache)
            if (c->rns_base == base && c->digits == digits) return *c;
        gadget_bconv_cache.push_back(std::make_unique<GadgetBConvCache>(make_gadget_cache(base, digits)));
        return *gadget_bconv_cache.back();
    }
    /// src/ring.rs:1730-1807
    GadgetBConvCache make_gadget_cache(const Base& base, const std::vector<std::pair<size_t, size_t>>& digits) {
        size_t r = base.size(), d = digits.size();
        ORACLE_ASSERT(d > 0, "digits");
        for (size_t i = 0; i < d; i++) {
            ORACLE_ASSERT(digits[i].first < digits[i].second && digits[i].second <= r, "digit range");
            if (i > 0) ORACLE_ASSERT(digits[i - 1].second <= digits[i].first, "digits must be sorted and disjoint");
        }
        int64_t max_p = 0, min_p = INT64_MAX;
        for (size_t i : base) max_p = std::max(max_p, rns_factors[i].p), min_p = std::min(min_p, rns_factors[i].p);
        size_t max_digit_len = 0;
        for (auto& dg : digits) max_digit_len = std::max(max_digit_len, dg.second - dg.first);
        GadgetBConvCache c;
        c.rns_base = base;
        c.digits = digits;
        size_t l2 = 0;
        for (u128 v = (u128)(4 * (i128)max_digit_len * max_p + 1); v; v >>= 1) l2++;
        c.log2_qtilde = std::max<size_t>(64, l2);
        i128 qtilde = (i128)1 << c.log2_qtilde;
        i128 cvmax = (qtilde - 1) / min_p + 1;
        ORACLE_ASSERT(cvmax <= INT64_MAX, "coefficients of correction vector don't fit into an i64");
        c.acc_before_reduce = (size_t)(I128_MAX / ((i128)max_p * max_p));
        // D_i / p_u mod q for any prime q: product of the digit's other primes
        auto digit_over_p = [&](size_t di, size_t u, int64_t q) {
            int64_t v = 1;
            for (size_t l = digits[di].first; l < digits[di].second; l++)
                if (l != u) v = rmul_mod(v, rns_factors[base[l]].p % q, q);
            return rem_euclid64(v, q);
        };
        auto digit_mod = [&](size_t di, int64_t q) {
            int64_t v = 1;
            for (size_t l = digits[di].first; l < digits[di].second; l++) v = rmul_mod(v, rns_factors[base[l]].p % q, q);
            return rem_euclid64(v, q);
        };
        std::vector<int64_t> dinv(r, 0);
        for (size_t di = 0; di < d; di++)
            for (size_t u = digits[di].first; u < digits[di].second; u++) {
                int64_t pu = rns_factors[base[u]].p;
                dinv[u] = smallest_lift(inv_mod_prime(digit_over_p(di, u, pu), pu), pu);
            }
        c.d_over_p_inv = import_tensor(dinv, Shape{1, r, 1, 1});
        std::vector<int64_t> mat(d * (r + 1) * r, 0), dmp;
        for (size_t di = 0; di < d; di++) {
            for (size_t j = 0; j < r; j++) {
                int64_t pj = rns_factors[base[j]].p;
                int64_t r_sqr = rem_euclid64(rmul_mod(mont_repr(1, pj), mont_repr(1, pj), pj), pj);
                for (size_t u = digits[di].first; u < digits[di].second; u++)
                    mat[(di * (r + 1) + j) * r + u] = smallest_lift(rmul_mod(digit_over_p(di, u, pj), r_sqr, pj), pj);
                int64_t neg_r = rem_euclid64(-mont_repr(1, pj), pj);
                dmp.push_back(smallest_lift(rmul_mod(digit_mod(di, pj), neg_r, pj), pj));
            }
            for (size_t u = digits[di].first; u < digits[di].second; u++)
                mat[(di * (r + 1) + r) * r + u] = (int64_t)rounded_div(qtilde, (i128)rns_factors[base[u]].p);
        }
        c.matrix = import_tensor(mat, Shape{d, r + 1, r, 1});
        c.d_mod_p = import_tensor(dmp, Shape{d, r, 1, 1});
        return c;
    }
    /// src/ring.rs:1809-1851
    void bconv_gadget_tensors(V64 dst, V64 src, const Base& base, const std::vector<std::pair<size_t, size_t>>& digits) {
        GadgetBConvCache& c = gadget_cache_for(base, digits);
        size_t r = base.size(), d = digits.size();
        ORACLE_ASSERT(src.shape == (Shape{1, r, src.shape[2], src.shape[3]}), "gadget src shape");
        ORACLE_ASSERT(dst.shape == (Shape{d, r, src.shape[2], src.shape[3]}), "gadget dst shape");
        Mods mods = mods_for(base);
        backend.hal_mul_mont64(src, c.d_over_p_inv.view(), mods);
        Tensor<i128> correction = backend.hal_allocate_i128(Shape{d, 1, src.shape[2], src.shape[3]});
        Tensor<i128> tmp = backend.hal_allocate_i128(Shape{d, r + 1, src.shape[2], src.shape[3]});
        for (size_t u = 0, chunk = 0; u < r; u += c.acc_before_reduce, chunk++) {
            size_t e = std::min(u + c.acc_before_reduce, r);
            backend.hal_matmul_i64(tmp.view(), c.matrix.view().slice(0, d, 0, r + 1, u, e, 0, 1),
                                   src.slice(0, 1, u, e, 0, src.shape[2], 0, src.shape[3]));
            V128 vals = tmp.view().base_range(0, r), corr = tmp.view().base_range(r, r + 1);
            if (chunk == 0) {
                backend.hal_red_mont64_double(dst, vals, mods);
                backend.hal_assign_i128(correction.view(), corr);
            } else {
                backend.hal_add_red_mont64_double(dst, vals, mods);
                backend.hal_add_i128(correction.view(), corr);
            }
        }
        backend.hal_bconv_correct_mont64(dst, correction.view(), c.d_mod_p.view(), mods, c.log2_qtilde);
        backend.hal_i64_to_mont64(dst, mods);
    }
};

}  // namespace oracle
