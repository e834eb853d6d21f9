// Oracle (test infrastructure only): CPU restatement of the dBFV pieces of the homomorphic CRT
// transform's baby-step / giant-step step, over the restated hal::cpu backend:
//   DBFVModulus, balanced_digits_vec             cyclosubfield-dbfv/src/dbfv.rs:56-121
//   DBFVAccumulator, allocate / add               src/dbfv.rs:124-163
//   fma / inner product with L' elements          src/dbfv.rs:193-260, 291-399
//   finish_accumulator, hom_fma_element_lprime    src/dbfv.rs:401-453
//   bsgs_split, pow_mod_m, galois elements        src/bootstrap/homcrt.rs:322-367
//   hom_cyclic_transform_dbfv                     src/bootstrap/homcrt.rs:369-429
//   SplitOverflowData, split_overflow              src/dbfv.rs:735-950
//   dbfv_reduce, dbfv_hom_mul, dbfv_mul_convolve   src/dbfv.rs:968-1143
//   dbfv_enc, dbfv_dec                             src/dbfv.rs:602-722
// Big-integer constants (Q mod 2^k, (Q/p) mod 2^k, round(Q/t) mod p) are evaluated without big
// integers: modulo 2^128 by wrapping i128 products, modulo p by products of residues.
#pragma once
#include "bfv.hpp"

namespace oracle {

/// src/dbfv.rs:56-81: t = 2^log2_t with digit base b = 2^log2_b
struct DBFVModulus {
    size_t log2_b, log2_t;
    size_t digits() const { return (log2_t - 1) / log2_b + 1; }
    i128 b() const { return (i128)1 << log2_b; }
};

/// src/dbfv.rs:97-121
inline std::vector<std::vector<i128>> balanced_digits_vec(const std::vector<i128>& x, i128 b, size_t max_digits) {
    std::vector<std::vector<i128>> result;
    std::vector<i128> current = x;
    for (size_t it = 0; it < max_digits; it++) {
        bool all_zero = true;
        for (i128 v : current) all_zero = all_zero && v == 0;
        if (all_zero) break;
        std::vector<i128> rems;
        for (i128& v : current) {
            i128 rem = cmod(v, b);
            rems.push_back(rem);
            v = (v - rem) / b;
        }
        result.push_back(rems);
    }
    return result;
}

/// src/dbfv.rs:124-150
struct DBFVAccumulator {
    WideRingEls acc;
    DBFVModulus modulus;
    Basis basis;
    size_t used_digits = 0;
    size_t capacity() const { return modulus.digits(); }
};

struct Dbfv {
    RingContext& ring;

    size_t digit_count(const RingView& ct) const {
        ORACLE_ASSERT(ct.count() % 2 == 0, "dBFV ciphertext rows");
        return ct.count() / 2;
    }
    DBFVAccumulator allocate_accumulator(DBFVModulus m, const Base& base, Basis basis) {
        return DBFVAccumulator{ring.allocate_wide(2 * m.digits(), base), m, basis, 0};
    }
    /// src/dbfv.rs:153-163
    void acc_add(DBFVAccumulator& acc, const RingView& ct) {
        size_t d = digit_count(ct);
        if (d == 0) return;
        ORACLE_ASSERT(d <= acc.capacity() && acc.basis == ct.basis && acc.acc.rns_base == ct.rns_base, "acc_add");
        acc.acc.add(ring.backend, 0, 2 * d, ct.data, ct.bound);
        acc.used_digits = std::max(acc.used_digits, d);
    }
    std::vector<Tensor<int64_t>> lprime_digit_tensors(const DBFVAccumulator& acc, const std::vector<i128>& rhs) {
        std::vector<Tensor<int64_t>> out;
        for (auto& coeffs : balanced_digits_vec(rhs, acc.modulus.b(), acc.modulus.digits()))
            out.push_back(ring.lprime_element_tensor(acc.acc.rns_base, coeffs));
        return out;
    }
    /// src/dbfv.rs:193-224
    void acc_fma_tensors(DBFVAccumulator& acc, const RingView& lhs, const std::vector<Tensor<int64_t>>& rhs) {
        size_t ld = digit_count(lhs);
        if (ld == 0 || rhs.empty()) return;
        ORACLE_ASSERT(ld <= acc.capacity() && acc.basis == lhs.basis && acc.acc.rns_base == lhs.rns_base, "acc_fma");
        size_t new_digits = std::min(acc.capacity(), ld + rhs.size() - 1);
        for (size_t i = 0; i < ld; i++)
            for (size_t j = 0; j < rhs.size(); j++) {
                size_t k = i + j;
                if (k < new_digits)
                    acc.acc.fma(ring.backend, 2 * k, 2 * k + 2, lhs.data.rows(2 * i, 2 * i + 2), lhs.bound,
                                rhs[j].view(), 1);
            }
        acc.used_digits = std::max(acc.used_digits, new_digits);
    }
    /// src/dbfv.rs:291-352
    void acc_inner_product_tensors(DBFVAccumulator& acc,
                                   const std::vector<std::pair<RingView, std::vector<Tensor<int64_t>>>>& terms) {
        size_t cap = acc.capacity(), max_new = 0;
        for (auto& t : terms) {
            size_t ld = digit_count(t.first);
            if (ld == 0 || t.second.empty()) continue;
            ORACLE_ASSERT(ld <= cap && acc.basis == t.first.basis && acc.acc.rns_base == t.first.rns_base,
                          "acc_inner_product");
            max_new = std::max(max_new, std::min(cap, ld + t.second.size() - 1));
        }
        if (max_new == 0) return;
        for (size_t k = 0; k < max_new; k++) {
            std::vector<std::tuple<V64, u128, V64, u128>> kt;
            for (auto& t : terms) {
                size_t ld = digit_count(t.first);
                if (ld == 0 || t.second.empty()) continue;
                size_t new_digits = std::min(cap, ld + t.second.size() - 1);
                if (k >= new_digits) continue;
                for (size_t j = 0; j < t.second.size(); j++) {
                    if (k < j) break;
                    size_t i = k - j;
                    if (i >= ld) continue;
                    kt.emplace_back(t.first.data.rows(2 * i, 2 * i + 2), t.first.bound, t.second[j].view(), 1);
                }
            }
            if (!kt.empty()) acc.acc.inner_product(ring.backend, 2 * k, 2 * k + 2, kt);
        }
        acc.used_digits = std::max(acc.used_digits, max_new);
    }
    /// src/dbfv.rs:401-404
    RingEls finish(const DBFVAccumulator& acc) { return ring.reduce_wide_rows(acc.acc, 0, 2 * acc.used_digits, acc.basis); }
    RingEls empty(const Base& base, Basis basis) { return ring.allocate_in_basis(0, base, basis); }
    /// src/dbfv.rs:431-453
    RingEls hom_fma_element_lprime(DBFVModulus m, const RingView& lhs, const std::vector<i128>& rhs,
                                   const RingView& summand) {
        ORACLE_ASSERT(lhs.basis == Basis::CRTBasis && summand.basis == Basis::CRTBasis, "CRT basis required");
        bool all_zero = true;
        for (i128 v : rhs) all_zero = all_zero && v == 0;
        if (digit_count(lhs) == 0 || all_zero) return ring.clone_els(summand);
        DBFVAccumulator acc = allocate_accumulator(m, lhs.rns_base, Basis::CRTBasis);
        acc_add(acc, summand);
        acc_fma_tensors(acc, lhs, lprime_digit_tensors(acc, rhs));
        return finish(acc);
    }
};

/// src/bootstrap/homcrt.rs:335-339
inline std::pair<size_t, size_t> bsgs_split(size_t len) {
    const size_t UNHOISTED_OVERHEAD = 3;  // homcrt.rs:333
    size_t best = 1, best_cost = (size_t)-1;
    for (size_t count = 1; count <= len; count++) {
        size_t cost = count + UNHOISTED_OVERHEAD * ((len - 1) / count + 1);
        if (cost < best_cost) best_cost = cost, best = count;
    }
    return {best, (len - 1) / best + 1};
}

/// src/bootstrap/homcrt.rs:341-347
inline uint64_t pow_mod_m(uint64_t g, size_t e, uint64_t m) {
    uint64_t r = 1;
    for (size_t i = 0; i < e; i++) r = (uint64_t)((u128)r * g % m);
    return r;
}

/// The Galois elements one cyclic transform of length `len` by `g` needs (homcrt.rs:350-361).
inline std::vector<uint64_t> transform_galois_elements(uint64_t g, size_t len, uint64_t m) {
    std::vector<uint64_t> out;
    if (len <= 1) return out;
    auto sp = bsgs_split(len);
    for (size_t j = 1; j < sp.first; j++) out.push_back(pow_mod_m(g, j, m));
    if (sp.second > 1) out.push_back(pow_mod_m(g, sp.first, m));
    return out;
}

/// src/bootstrap/homcrt.rs:369-429: Σ_i coeffs[i] σ^i(ct) with baby steps sharing the gadget
/// decomposition and giant steps applying one unhoisted automorphism to the accumulated result.
/// `key_for(g)` returns the Galois key of automorphism g.
inline RingEls hom_cyclic_transform_dbfv(RingContext& ring, DBFVModulus modulus, uint64_t automorphism,
                                         const std::vector<std::vector<i128>>& coeffs, const RingView& ct,
                                         const std::function<const KeySwitchKey*(uint64_t)>& key_for) {
    Dbfv D{ring};
    uint64_t st = 0;
    Bfv bfv(ring, &st);
    const size_t len = coeffs.size();
    const Base base = ct.rns_base;
    if (len == 0) return D.empty(base, Basis::CRTBasis);
    if (len == 1) {
        RingEls summand = D.empty(base, Basis::CRTBasis);
        return D.hom_fma_element_lprime(modulus, ct, coeffs[0], as_view(summand));
    }
    auto sp = bsgs_split(len);
    const size_t baby_steps = sp.first, giant_steps = sp.second;
    const uint64_t m = ring.field.m;
    const size_t d = D.digit_count(ct);
    std::vector<uint64_t> baby_exps;
    std::vector<const KeySwitchKey*> baby_keys;
    for (size_t j = 1; j < baby_steps; j++) {
        baby_exps.push_back(pow_mod_m(automorphism, j, m));
        baby_keys.push_back(key_for(baby_exps.back()));
    }
    std::vector<RingEls> babys;
    babys.push_back(ring.clone_els(ct));
    for (size_t j = 1; j < baby_steps; j++) babys.push_back(ring.allocate_in_basis(2 * d, base, Basis::CRTBasis));
    for (size_t di = 0; di < d; di++) {
        std::vector<RingEls> rot = bfv.bfv_hom_gal(as_view(babys[0]).rows(2 * di, 2 * di + 2), baby_exps, baby_keys);
        for (size_t j = 0; j < rot.size(); j++)
            ring.backend.hal_assign(babys[j + 1].data.view().rows(2 * di, 2 * di + 2), rot[j].data.view());
    }
    const uint64_t giant_exp = pow_mod_m(automorphism, baby_steps, m);
    RingEls out = D.empty(base, Basis::CRTBasis);
    for (size_t giant = giant_steps; giant-- > 0;) {
        if (giant != giant_steps - 1) {
            size_t od = D.digit_count(as_view(out));
            RingEls rotated = ring.allocate_in_basis(2 * od, base, Basis::CRTBasis);
            for (size_t di = 0; di < od; di++) {
                std::vector<RingEls> r =
                    bfv.bfv_hom_gal(as_view(out).rows(2 * di, 2 * di + 2), {giant_exp}, {key_for(giant_exp)});
                ring.backend.hal_assign(rotated.data.view().rows(2 * di, 2 * di + 2), r[0].data.view());
            }
            out = std::move(rotated);
        }
        DBFVAccumulator acc = D.allocate_accumulator(modulus, base, Basis::CRTBasis);
        std::vector<std::pair<RingView, std::vector<Tensor<int64_t>>>> terms;
        size_t nt = std::min(baby_steps, len - giant * baby_steps);
        for (size_t j = 0; j < nt; j++)
            terms.emplace_back(as_view(babys[j]), D.lprime_digit_tensors(acc, coeffs[giant * baby_steps + j]));
        D.acc_inner_product_tensors(acc, terms);
        D.acc_add(acc, as_view(out));
        out = D.finish(acc);
    }
    return out;
}

/// rows [s, e) of dimension 1
inline V64 dim1(V64 v, size_t s, size_t e) { return v.slice(0, v.shape[0], s, e, 0, v.shape[2], 0, v.shape[3]); }

/// src/hal/mod.rs:71-76
inline std::pair<int64_t, int64_t> split_i128_limbs(i128 x) {
    int64_t lo = (int64_t)x;
    int64_t hi = (int64_t)((x - (i128)lo) >> 64);
    return {lo, hi};
}

/// src/dbfv.rs:762-768
inline i128 inv_mod_2_128(i128 q) {
    u128 x = (u128)q, qq = (u128)q;
    for (int i = 0; i < 6; i++) x = x * (2 - qq * x);
    return (i128)x;
}

/// Q mod 2^128 (wrapping product of the base's primes)
inline u128 q_mod_2_128(const RingContext& ring, const Base& base) {
    u128 q = 1;
    for (size_t i : base) q *= (u128)ring.prime(i);
    return q;
}

/// round(Q / 2^k) modulo p, for 1 <= k <= 126 (feanor rounded_div; Q odd, so no ties)
inline BigResidue delta_pow2_residue(const RingContext& ring, const Base& base, size_t k) {
    const u128 mask = ((u128)1 << k) - 1;
    const u128 c = q_mod_2_128(ring, base) & mask;
    const int64_t extra = c >= ((u128)1 << (k - 1)) ? 1 : 0;
    return [c, k, extra](int64_t p) -> int64_t {
        int64_t cp = (int64_t)(c % (u128)p);
        int64_t two_k = rpow_mod(2, (uint64_t)k, p);
        int64_t v = rmul_mod(rem_euclid64(-cp, p), inv_mod_prime(two_k, p), p);
        return rem_euclid64(v + extra, p);
    };
}

/// src/ring.rs:907-920: mont(mont(smallest lift of x mod p))
inline Tensor<int64_t> scalar_tensor_big_mont2(const RingContext& ring, const Base& base, const BigResidue& x) {
    std::vector<int64_t> v;
    for (size_t i : base) {
        int64_t p = ring.prime(i);
        v.push_back(mont_repr(mont_repr(smallest_lift(x(p), p), p), p));
    }
    return ring.import_tensor(v, Shape{1, base.size(), 1, 1});
}

/// src/dbfv.rs:735-849
struct SplitOverflowData {
    size_t log2_b, log2_t, log2_r, log2_gamma;
    Tensor<int64_t> r_q_over_p_inv, matrix;
    i128 neg_q_inv_mod_r, q_mod_r;
    std::vector<Tensor<int64_t>> neg_b_delta_mont2;
    size_t limbs() const { return log2_r <= 62 ? 1 : 2; }

    SplitOverflowData(const RingContext& ring, DBFVModulus m, const Base& base) {
        log2_b = m.log2_b, log2_t = m.log2_t;
        log2_r = m.log2_t - m.log2_b;
        ORACLE_ASSERT(log2_r >= 1 && log2_r <= 126, "t/b must be between 2 and 2^126");
        const size_t L = limbs();
        const u128 rmask = ((u128)1 << log2_r) - 1;
        int64_t max_p = 0, min_p = INT64_MAX;
        for (size_t i : base) max_p = std::max(max_p, ring.prime(i)), min_p = std::min(min_p, ring.prime(i));
        u128 x = 4 * (u128)base.size() * (u128)max_p + 1;
        size_t bits = 0;
        while ((x >> bits) > 0) bits++;
        log2_gamma = std::max<size_t>(64, bits);
        ORACLE_ASSERT(log2_gamma <= 126, "split overflow precision");
        const i128 gamma = (i128)1 << log2_gamma;
        std::vector<int64_t> mat;
        std::vector<i128> qpr;
        for (size_t i : base) {
            u128 q = 1;
            for (size_t j : base)
                if (j != i) q *= (u128)ring.prime(j);
            qpr.push_back((i128)(q & rmask));
        }
        for (i128 c : qpr) mat.push_back(split_i128_limbs(c).first);
        if (L == 2)
            for (i128 c : qpr) mat.push_back(split_i128_limbs(c).second);
        for (size_t i : base) mat.push_back((int64_t)rounded_div(gamma, (i128)ring.prime(i)));
        matrix = ring.import_tensor(mat, Shape{1, L + 1, base.size(), 1});
        q_mod_r = (i128)(q_mod_2_128(ring, base) & rmask);
        i128 ninv = -inv_mod_2_128(q_mod_r);
        neg_q_inv_mod_r = (i128)((u128)ninv & rmask);
        r_q_over_p_inv = ring.q_over_p_inv_tensor(base, (i128)1 << log2_r);
        BigResidue delta = delta_pow2_residue(ring, base, m.log2_t);
        for (size_t k = 0; k < L; k++) {
            size_t lb = m.log2_b;
            BigResidue f = [delta, lb, k](int64_t p) -> int64_t {
                int64_t v = rmul_mod(delta(p), rpow_mod(2, (uint64_t)lb, p), p);
                v = rmul_mod(v, rpow_mod(2, 64 * (uint64_t)k, p), p);
                return rem_euclid64(-v, p);
            };
            neg_b_delta_mont2.push_back(scalar_tensor_big_mont2(ring, base, f));
        }
    }
};

/// src/dbfv.rs:891-950: x <- x_lo in place, returns the overflow limbs [count, limbs, ...]
inline Tensor<int64_t> split_overflow(RingContext& ring, const SplitOverflowData& data, V64 x, u128 x_bound,
                                      const Base& base) {
    const CpuBackend& be = ring.backend;
    Shape shape{x.shape[0], x.shape[1], x.shape[2], x.shape[3]};
    ORACLE_ASSERT(shape[1] == base.size(), "split_overflow base");
    const size_t L = data.limbs();
    Mods mods = ring.mods_for(base);
    Tensor<int64_t> lifts = be.hal_allocate_i64(shape);
    be.hal_assign(lifts.view(), x);
    be.hal_mul_mont64(lifts.view(), data.r_q_over_p_inv.view(), mods);
    Tensor<i128> sums = be.hal_allocate_i128(Shape{shape[0], L + 1, shape[2], shape[3]});
    be.hal_matmul_i64(sums.view(), data.matrix.view(), lifts.view());
    Tensor<int64_t> overflow = be.hal_allocate_i64(Shape{shape[0], L, shape[2], shape[3]});
    if (L == 1)
        be.hal_bconv_correct_pow2(overflow.view(), sums.view(), (int64_t)data.q_mod_r, (int64_t)data.neg_q_inv_mod_r,
                                  data.log2_gamma, data.log2_r);
    else
        be.hal_bconv_correct_pow2_wide(overflow.view(), sums.view(), data.q_mod_r, data.neg_q_inv_mod_r,
                                       data.log2_gamma, data.log2_r);
    WideRingEls acc = ring.allocate_wide(shape[0], base);
    for (size_t k = 0; k < L; k++)
        acc.fma_unbounded(be, 0, acc.count(), dim1(overflow.view(), k, k + 1), data.neg_b_delta_mont2[k].view());
    acc.add(be, 0, acc.count(), x, x_bound);
    ring.reduce_wide_tensor(x, acc, 0, acc.count());
    return overflow;
}

/// src/dbfv.rs:968-1032 (period basis in and out)
inline RingEls dbfv_reduce(RingContext& ring, DBFVModulus m, const RingView& ct) {
    Dbfv D{ring};
    const size_t d = D.digit_count(ct);
    ORACLE_ASSERT(d <= m.digits(), "dbfv_reduce digits");
    if (m.digits() == 1 || d == 0) return ring.clone_els(ct);
    ORACLE_ASSERT(ct.basis == Basis::PeriodBasis, "dbfv_reduce basis");
    const Base base = ct.rns_base;
    SplitOverflowData data(ring, m, base);
    BigResidue delta = delta_pow2_residue(ring, base, m.log2_t);
    std::vector<Tensor<int64_t>> delta_mont2;
    for (size_t k = 0; k < data.limbs(); k++) {
        BigResidue f = [delta, k](int64_t p) { return rmul_mod(delta(p), rpow_mod(2, 64 * (uint64_t)k, p), p); };
        delta_mont2.push_back(scalar_tensor_big_mont2(ring, base, f));
    }
    RingEls result = ring.allocate(2 * m.digits(), base);
    ring.backend.hal_assign(result.data.view().rows(0, 2 * d), ct.data);
    bool have_carry = false;
    Tensor<int64_t> carry;
    for (size_t i = 0; i < m.digits(); i++) {
        u128 input_row_bound = i < d ? ct.bound : 1;
        V64 rows = result.data.view().rows(2 * i, 2 * i + 2);
        if (have_carry) {
            WideRingEls acc = ring.allocate_wide(2, base);
            for (size_t k = 0; k < delta_mont2.size(); k++)
                acc.fma_unbounded(ring.backend, 0, 2, dim1(carry.view(), k, k + 1), delta_mont2[k].view());
            acc.add(ring.backend, 0, 2, rows, input_row_bound);
            ring.reduce_wide_tensor(rows, acc, 0, 2);
        }
        u128 row_bound = have_carry ? 1 : input_row_bound;
        carry = split_overflow(ring, data, rows, row_bound, base);
        have_carry = true;
    }
    result.bound = 1;
    return result;
}

/// src/dbfv.rs:1081-1143
inline RingEls dbfv_mul_convolve(RingContext& ring, Bfv& bfv, DBFVModulus m, const RingEls& lhs, const RingEls& rhs,
                                 size_t base_len, const KeySwitchKey& rk, Basis output_basis) {
    Dbfv D{ring};
    const size_t d1 = D.digit_count(as_view(lhs)), d2 = D.digit_count(as_view(rhs));
    const size_t d_out = std::min(m.digits(), d1 + d2 - 1);
    WideRingEls acc = ring.allocate_wide(3 * d_out, lhs.rns_base);
    for (size_t k = 0; k < d_out; k++) {
        std::vector<std::tuple<V64, u128, V64, u128>> t0, t1, t2;
        const size_t jlo = k >= d2 - 1 ? k - (d2 - 1) : 0, jhi = std::min(k, d1 - 1);
        for (size_t j = jlo; j <= jhi; j++) {
            V64 l0 = lhs.data.view().rows(2 * j, 2 * j + 1), l1 = lhs.data.view().rows(2 * j + 1, 2 * j + 2);
            V64 r0 = rhs.data.view().rows(2 * (k - j), 2 * (k - j) + 1);
            V64 r1 = rhs.data.view().rows(2 * (k - j) + 1, 2 * (k - j) + 2);
            t0.emplace_back(l0, lhs.bound, r0, rhs.bound);
            t1.emplace_back(l0, lhs.bound, r1, rhs.bound);
            t1.emplace_back(l1, lhs.bound, r0, rhs.bound);
            t2.emplace_back(l1, lhs.bound, r1, rhs.bound);
        }
        acc.inner_product(ring.backend, 3 * k, 3 * k + 1, t0);
        acc.inner_product(ring.backend, 3 * k + 1, 3 * k + 2, t1);
        acc.inner_product(ring.backend, 3 * k + 2, 3 * k + 3, t2);
    }
    RingEls prod = ring.reduce_wide(acc, Basis::CRTBasis);
    ring.crt_to_pb(prod);
    RingEls rescaled = bfv.rescale_to_base(std::move(prod), base_len, ((i128)1) << m.log2_t);
    RingEls result = ring.allocate_in_basis(2 * d_out, rescaled.rns_base, output_basis);
    for (size_t k = 0; k < d_out; k++) {
        RingEls rl = bfv.relin(as_view(rescaled).rows(3 * k, 3 * k + 3), rk, output_basis);
        ring.backend.hal_assign(result.data.view().rows(2 * k, 2 * k + 2), rl.data.view());
        result.bound = rl.bound;
    }
    return result;
}

/// src/dbfv.rs:661-689: CRT basis, all digits
inline RingEls dbfv_enc(RingContext& ring, Bfv& bfv, DBFVModulus m, const Base& base, const std::vector<i128>& ptxt,
                        const RingEls& sk, double log2_alpha) {
    const size_t digits = m.digits();
    const double la = log2_alpha + (double)(m.log2_b * (digits - 1));  // src/dbfv.rs:602-604
    RingEls digit0 = bfv.bfv_enc(base, ((i128)1) << m.log2_t, ptxt, sk, la);
    if (digits == 1) return digit0;
    RingEls ct = ring.allocate_in_basis(2 * digits, base, Basis::CRTBasis);
    ring.backend.hal_assign(ct.data.view().rows(0, 2), digit0.data.view());
    for (size_t i = 1; i < digits; i++) {
        RingEls z = bfv.bfv_enc_zero(base, sk, la);
        ring.backend.hal_assign(ct.data.view().rows(2 * i, 2 * i + 2), z.data.view());
    }
    ring.crt_to_pb(ct);
    RingEls result = dbfv_reduce(ring, m, as_view(ct));
    ring.pb_to_crt(result);
    return result;
}

/// src/dbfv.rs:1034-1059 (both operands in period basis)
inline RingEls dbfv_hom_mul(RingContext& ring, Bfv& bfv, DBFVModulus m, const RingView& lhs, const RingView& rhs,
                            const KeySwitchKey& rk, Basis output_basis) {
    Dbfv D{ring};
    RingEls lr = dbfv_reduce(ring, m, lhs), rr = dbfv_reduce(ring, m, rhs);
    if (D.digit_count(as_view(lr)) == 0) return lr;
    if (D.digit_count(as_view(rr)) == 0) return rr;
    const size_t base_len = lr.rns_base.size();
    RingEls ll = bfv.lift_to_extended(as_view(lr), nullptr), rl = bfv.lift_to_extended(as_view(rr), nullptr);
    return dbfv_mul_convolve(ring, bfv, m, ll, rl, base_len, rk, output_basis);
}

}  // namespace oracle
