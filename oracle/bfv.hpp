// ORACLE — test infrastructure only (see arith.hpp). Restates the BFV layer of
// cyclosubfield-dbfv/src/bfv.rs that drives the hot path:
//   clip_digits, sigma/alpha            src/bfv.rs:120-167
//   sample_gaussian, gen_sk, add_error  src/bfv.rs:170-204
//   random_element, encode              src/bfv.rs:207-247
//   enc_zero, enc, finish_enc           src/bfv.rs:277-326
//   noisy_plaintext (decryption core)   src/bfv.rs:330-343
//   select_digits, gadget_decompose     src/bfv.rs:388-426
//   gen_ksk, gen_rk, gen_gk             src/bfv.rs:433-491
//   key_switch_acc, key_switch          src/bfv.rs:498-556
//   lift_to_extended, rescale_to_base   src/bfv.rs:564-622
//   mod_switch_down                     src/bfv.rs:628-662
//   hom_mul_raw_acc, relin, hom_mul     src/bfv.rs:667-775
//   bfv_hom_gal                         src/bfv.rs:783-841
//   splitmix64                          src/bfv.rs:880-886
// Plaintext decoding (big-integer CRT reconstruction, src/bfv.rs:249-271) is done by the Python
// test code from the exported period-basis residues.
#pragma once
#include "ring.hpp"

namespace oracle {

static const size_t SK_HWT = 128;       // src/bfv.rs:41
static const double MIN_SIGMA = 3.2;    // src/bfv.rs:139

/// src/bfv.rs:880-886
inline uint64_t splitmix64(uint64_t* state) {
    *state += 0x9E3779B97F4A7C15ull;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef std::vector<std::pair<size_t, size_t>> Digits;

/// src/bfv.rs:120-126
inline Digits clip_digits(const Digits& digits, size_t base_len) {
    Digits r;
    for (auto& d : digits)
        if (d.first < base_len) r.push_back({d.first, std::min(d.second, base_len)});
    return r;
}
/// src/bfv.rs:388-400
inline Digits select_digits(size_t digits, size_t rns_base_len) {
    ORACLE_ASSERT(digits <= rns_base_len, "too many gadget digits");
    size_t per_small = rns_base_len / digits, large = rns_base_len % digits, current = 0;
    Digits r;
    for (size_t i = 0; i < digits; i++) {
        size_t len = i < large ? per_small + 1 : per_small;
        r.push_back({current, current + len});
        current += len;
    }
    return r;
}

/// A key switching key (src/bfv.rs:56-64): one size-2 CRT-basis batch per digit.
struct KeySwitchKey {
    Digits digits;
    std::vector<RingEls> keys;
};

struct Bfv {
    RingContext& ring;
    uint64_t* rng_state;
    explicit Bfv(RingContext& r, uint64_t* state) : ring(r), rng_state(state) {}
    uint64_t rng() { return splitmix64(rng_state); }

    /// src/bfv.rs:149-160
    double sigma_for_log2_alpha(const Base& base, double log2_alpha) const {
        double log2_sigma = ring.log2_modulus_of(base) - log2_alpha;
        return std::fmax(MIN_SIGMA, std::exp2(log2_sigma));
    }
    /// src/bfv.rs:165-167
    double log2_alpha_for_sigma(const Base& base, double sigma) const { return ring.log2_modulus_of(base) - std::log2(sigma); }

    /// src/bfv.rs:170-175
    i128 sample_gaussian(double sigma) {
        double u1 = ((double)(rng() >> 11) + 0.5) / (double)(1ull << 53);
        double u2 = (double)(rng() >> 11) / (double)(1ull << 53);
        double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
        return (i128)std::round(g * sigma);
    }
    /// src/bfv.rs:180-190
    RingEls gen_sk() {
        size_t n = ring.n();
        std::vector<i128> coeffs(n, 0);
        for (size_t i = 0; i < SK_HWT; i++) {
            size_t j = (size_t)(rng() % (uint64_t)n);
            coeffs[j] = (i128)(rng() % 2) * 2 - 1;
        }
        RingEls sk = ring.element_from_pb_coeffs(ring.initial_rns_base(), coeffs);
        ring.pb_to_crt(sk);
        return sk;
    }
    /// src/bfv.rs:195-204
    void add_error(RingEls& els, double sigma) {
        ORACLE_ASSERT(els.basis == Basis::PeriodBasis && els.count() == 1, "add_error operand");
        std::vector<i128> coeffs;
        for (size_t i = 0; i < ring.n(); i++) coeffs.push_back(sample_gaussian(sigma));
        RingEls error = ring.element_from_pb_coeffs(els.rns_base, coeffs);
        WideRingEls acc = ring.allocate_wide(1, els.rns_base);
        ring.add(acc, as_view(els));
        ring.add(acc, as_view(error));
        ring.reduce_wide_into(as_view(els), acc);
    }
    /// src/bfv.rs:207-222
    RingEls random_element(const Base& base) {
        std::vector<int64_t> values;
        for (size_t idx : base) {
            int64_t p = ring.prime(idx);
            for (size_t i = 0; i < ring.n(); i++) values.push_back((int64_t)(rng() % (uint64_t)p));
        }
        RingEls result = ring.allocate_in_basis(1, base, Basis::CRTBasis);
        ring.backend.hal_import(result.data.view(), values.data(), values.size());
        return result;
    }
    /// Delta = round(Q/t) modulo p (src/bfv.rs:244, feanor rounded_div: half away from zero).
    BigResidue delta_residue(const Base& base, u128 t) const {
        // Q mod t
        u128 q_mod_t = 1 % t;
        for (size_t i : base) q_mod_t = (u128)(((q_mod_t % t) * ((u128)ring.prime(i) % t)) % t);
        // floor((Q + floor(t/2)) / t) = (Q - c)/t + floor((c + floor(t/2))/t)
        u128 extra = (q_mod_t + t / 2) / t;
        return [q_mod_t, t, extra](int64_t p) -> int64_t {
            // (Q - c)/t mod p with Q = 0 mod p
            int64_t c = (int64_t)(q_mod_t % (u128)p);
            int64_t tinv = inv_mod_prime((int64_t)(t % (u128)p), p);
            int64_t v = rmul_mod(rem_euclid64(-c, p), tinv, p);
            return rem_euclid64(v + (int64_t)extra, p);
        };
    }
    /// src/bfv.rs:226-247
    RingEls encode_pb_scaled(const Base& base, i128 t, const std::vector<i128>& ptxt) {
        std::vector<i128> coeffs;
        for (i128 c : ptxt) coeffs.push_back(cmod(c, t));
        RingEls result = ring.element_from_pb_coeffs(base, coeffs);
        ring.mul_scalar_big(result, delta_residue(base, (u128)t));
        return result;
    }
    /// src/bfv.rs:310-326
    RingEls finish_enc(const Base& base, const RingEls& sk, RingEls b) {
        RingEls a = random_element(base);
        RingEls ct = ring.allocate_in_basis(2, base, Basis::CRTBasis);
        WideRingEls acc = ring.allocate_wide(1, base);
        ring.fma(acc, as_view(a), as_view(sk).restrict_base(base.size()));
        ring.add(acc, as_view(b));
        ring.reduce_wide_into(as_view(ct).rows(0, 1), acc);
        ring.mul_scalar(a, -1);
        ring.backend.hal_assign(ct.data.view().rows(1, 2), a.data.view());
        return ct;
    }
    /// src/bfv.rs:277-288
    RingEls bfv_enc_zero(const Base& base, const RingEls& sk, double log2_alpha) {
        RingEls b = ring.allocate(1, base);
        add_error(b, sigma_for_log2_alpha(base, log2_alpha));
        ring.pb_to_crt(b);
        return finish_enc(base, sk, std::move(b));
    }
    /// src/bfv.rs:294-307
    RingEls bfv_enc(const Base& base, i128 t, const std::vector<i128>& ptxt, const RingEls& sk, double log2_alpha) {
        RingEls b = encode_pb_scaled(base, t, ptxt);
        add_error(b, sigma_for_log2_alpha(base, log2_alpha));
        ring.pb_to_crt(b);
        return finish_enc(base, sk, std::move(b));
    }
    /// src/bfv.rs:330-343: c0 + c1 s in period basis.
    RingEls noisy_plaintext(const RingView& ct, const RingEls& sk) {
        ORACLE_ASSERT(ct.basis == Basis::CRTBasis && ct.count() == 2, "ciphertext");
        WideRingEls acc = ring.allocate_wide(1, ct.rns_base);
        ring.fma(acc, ct.rows(1, 2), as_view(sk).restrict_base(ct.rns_base.size()));
        ring.add(acc, ct.rows(0, 1));
        RingEls noisy = ring.reduce_wide(acc, Basis::CRTBasis);
        ring.crt_to_pb(noisy);
        return noisy;
    }
    /// src/bfv.rs:408-426
    RingEls gadget_decompose(const RingView& els, const Digits& digits) {
        ORACLE_ASSERT(els.basis == Basis::PeriodBasis && els.count() == 1, "gadget_decompose operand");
        ring.assert_mul_mont_safe(els.bound, els.rns_base);
        RingEls result = ring.allocate(digits.size(), els.rns_base);
        RingEls tmp = ring.clone_els(els);
        ring.bconv_gadget_tensors(result.data.view(), tmp.data.view(), els.rns_base, digits);
        ring.pb_to_crt(result);
        return result;
    }
    /// src/bfv.rs:433-458
    KeySwitchKey gen_ksk(const Base& base, const RingEls& old_sk, const RingEls& new_sk, const Digits& digits,
                         double log2_alpha) {
        KeySwitchKey k;
        k.digits = digits;
        for (auto& digit : digits) {
            RingEls ct = bfv_enc_zero(base, new_sk, log2_alpha);
            // factor = 1 modulo the digit's primes, 0 modulo the others
            std::map<int64_t, int64_t> residue;
            for (size_t j = 0; j < base.size(); j++)
                residue[ring.prime(base[j])] = (j >= digit.first && j < digit.second) ? 1 : 0;
            BigResidue factor = [residue](int64_t p) { return residue.at(p); };
            WideRingEls acc = ring.allocate_wide(1, base);
            ring.fma_scalar_big(acc, as_view(old_sk).restrict_base(base.size()), factor);
            ring.add(acc, as_view(ct).rows(0, 1));
            ring.reduce_wide_into(as_view(ct).rows(0, 1), acc);
            k.keys.push_back(std::move(ct));
        }
        return k;
    }
    /// src/bfv.rs:462-474
    KeySwitchKey gen_rk(const RingEls& sk, const Digits& digits, double log2_alpha) {
        Base base = ring.initial_rns_base();
        WideRingEls acc = ring.allocate_wide(1, base);
        ring.fma(acc, as_view(sk), as_view(sk));
        RingEls sk_sqr = ring.reduce_wide(acc, Basis::CRTBasis);
        return gen_ksk(base, sk_sqr, sk, digits, log2_alpha);
    }
    /// src/bfv.rs:479-491
    KeySwitchKey gen_gk(const RingEls& sk, uint64_t g, const Digits& digits, double log2_alpha) {
        Base base = ring.initial_rns_base();
        RingEls gal_sk = ring.allocate_in_basis(1, base, Basis::CRTBasis);
        ring.apply_galois(gal_sk, as_view(sk), g);
        return gen_ksk(base, gal_sk, sk, digits, log2_alpha);
    }
    /// src/bfv.rs:498-528
    void key_switch_acc(WideRingEls& acc, const RingView& c1_pb, const KeySwitchKey& ksk) {
        ORACLE_ASSERT(c1_pb.count() == 1 && c1_pb.basis == Basis::PeriodBasis, "key_switch_acc operand");
        size_t base_len = c1_pb.rns_base.size();
        Digits digits = clip_digits(ksk.digits, base_len);
        RingEls parts = gadget_decompose(c1_pb, digits);
        std::vector<std::tuple<V64, u128, V64, u128>> terms;
        for (size_t i = 0; i < digits.size(); i++) {
            RingView key = as_view(ksk.keys[i]).restrict_base(base_len);
            terms.emplace_back(parts.data.view().rows(i, i + 1), parts.bound, key.data, key.bound);
        }
        if (!terms.empty()) acc.inner_product(ring.backend, 0, 2, terms);
    }
    /// src/bfv.rs:533-556
    RingEls key_switch(const RingView& c0_crt, const RingView& c1_pb, const KeySwitchKey& ksk) {
        WideRingEls acc = ring.allocate_wide(2, c1_pb.rns_base);
        key_switch_acc(acc, c1_pb, ksk);
        acc.add(ring.backend, 0, 1, c0_crt.data, c0_crt.bound);
        return ring.reduce_wide(acc, Basis::CRTBasis);
    }
    /// src/bfv.rs:564-595
    RingEls lift_to_extended(const RingView& pb, const RingView* crt) {
        ORACLE_ASSERT(pb.basis == Basis::PeriodBasis && pb.bound <= 2, "lift operand");
        size_t base_len = pb.rns_base.size();
        Base extension = ring.extension_rns_base_for(pb.rns_base);
        Base lifted = pb.rns_base;
        lifted.insert(lifted.end(), extension.begin(), extension.end());
        RingEls result = ring.allocate(pb.count(), lifted);
        RingEls tmp = ring.clone_els(pb);
        V64 rv = result.data.view();
        ring.bconv_tensors(rv.base_range(base_len, lifted.size()), extension, tmp.data.view(), pb.rns_base);
        if (crt) {
            ring.pb_to_crt_tensor(rv.base_range(base_len, lifted.size()), extension);
            ring.backend.hal_assign(rv.base_range(0, base_len), crt->data);
            result.bound = crt->bound;
        } else {
            ring.backend.hal_assign(rv.base_range(0, base_len), pb.data);
            ring.pb_to_crt_tensor(rv, lifted);
        }
        result.basis = Basis::CRTBasis;
        return result;
    }
    /// src/bfv.rs:601-622
    RingEls rescale_to_base(RingEls x, size_t base_len, i128 t) {
        ORACLE_ASSERT(x.basis == Basis::PeriodBasis, "rescale operand");
        size_t count = x.count();
        Base base(x.rns_base.begin(), x.rns_base.begin() + base_len);
        Base extension(x.rns_base.begin() + base_len, x.rns_base.end());
        ring.mul_scalar(x, t);
        RingEls tmp = ring.allocate(count, extension);
        V64 xv = x.data.view();
        ring.bconv_tensors(tmp.data.view(), extension, xv.base_range(0, base_len), base);
        ring.backend.hal_sub_i64(xv.base_range(base_len, x.rns_base.size()), tmp.data.view());
        Base bcopy = base;
        const RingContext& rc = ring;
        Tensor<int64_t> q_inv =
            ring.inverse_scalar_tensor(extension, [&rc, bcopy](int64_t p) { return rc.modulus_mod(bcopy, p); });
        ring.backend.hal_mul_mont64(xv.base_range(base_len, x.rns_base.size()), q_inv.view(), ring.mods_for(extension));
        RingEls result = ring.allocate(count, base);
        ring.bconv_tensors(result.data.view(), base, xv.base_range(base_len, x.rns_base.size()), extension);
        return result;
    }
    /// src/bfv.rs:628-662
    RingEls mod_switch_down(const RingView& els, size_t new_len) {
        ORACLE_ASSERT(els.basis == Basis::PeriodBasis && new_len <= els.rns_base.size(), "mod_switch_down operand");
        Base kept(els.rns_base.begin(), els.rns_base.begin() + new_len);
        Base dropped(els.rns_base.begin() + new_len, els.rns_base.end());
        if (dropped.empty()) return ring.clone_els(els);
        RingEls dropped_part = ring.allocate(els.count(), dropped);
        ring.backend.hal_assign(dropped_part.data.view(), els.data.base_range(new_len, els.rns_base.size()));
        RingEls tmp = ring.allocate(els.count(), kept);
        ring.bconv_tensors(tmp.data.view(), kept, dropped_part.data.view(), dropped);
        RingEls result = ring.clone_els(els.restrict_base(new_len));
        ring.assert_mul_mont_safe(result.bound + 1, kept);
        ring.backend.hal_sub_i64(result.data.view(), tmp.data.view());
        const RingContext& rc = ring;
        Tensor<int64_t> inv =
            ring.inverse_scalar_tensor(kept, [&rc, dropped](int64_t p) { return rc.modulus_mod(dropped, p); });
        ring.backend.hal_mul_mont64(result.data.view(), inv.view(), ring.mods_for(kept));
        result.bound = 1;
        return result;
    }
    /// src/bfv.rs:667-683
    void hom_mul_raw_acc(WideRingEls& acc, size_t row, V64 lhs, V64 rhs) {
        V64 l0 = lhs.rows(0, 1), l1 = lhs.rows(1, 2), r0 = rhs.rows(0, 1), r1 = rhs.rows(1, 2);
        acc.fma(ring.backend, row, row + 1, l0, 1, r0, 1);
        acc.fma(ring.backend, row + 1, row + 2, l0, 1, r1, 1);
        acc.fma(ring.backend, row + 1, row + 2, l1, 1, r0, 1);
        acc.fma(ring.backend, row + 2, row + 3, l1, 1, r1, 1);
    }
    /// src/bfv.rs:699-741
    RingEls relin(RingView prod, const KeySwitchKey& rk, Basis output_basis) {
        ORACLE_ASSERT(prod.basis == Basis::PeriodBasis && prod.count() == 3, "relin operand");
        WideRingEls acc = ring.allocate_wide(2, prod.rns_base);
        RingView c2{prod.rns_base, Basis::PeriodBasis, prod.bound, prod.data.rows(2, 3)};
        key_switch_acc(acc, c2, rk);
        if (output_basis == Basis::CRTBasis) {
            ORACLE_ASSERT(prod.bound <= 2, "basis transforms require representatives bounded by 2p");
            ring.pb_to_crt_tensor(prod.data.rows(0, 2), prod.rns_base);
            acc.add(ring.backend, 0, 2, prod.data.rows(0, 2), 1);
            return ring.reduce_wide(acc, Basis::CRTBasis);
        }
        RingEls switched = ring.reduce_wide(acc, Basis::CRTBasis);
        ring.crt_to_pb(switched);
        RingView c0c1{prod.rns_base, Basis::PeriodBasis, prod.bound, prod.data.rows(0, 2)};
        ring.add_els(switched, c0c1);
        return switched;
    }
    /// src/bfv.rs:747-775
    RingEls bfv_hom_mul(i128 t, const RingEls& lhs, const RingEls& rhs, const KeySwitchKey& rk, Basis output_basis) {
        ORACLE_ASSERT(lhs.rns_base == rhs.rns_base && lhs.count() == 2 && rhs.count() == 2, "hom_mul operands");
        ORACLE_ASSERT(lhs.basis == Basis::CRTBasis && rhs.basis == Basis::CRTBasis, "hom_mul basis");
        size_t base_len = lhs.rns_base.size();
        auto lift = [&](const RingEls& ct) {
            RingEls ct_pb = ring.clone_els(as_view(ct));
            ring.crt_to_pb(ct_pb);
            RingView crt = as_view(ct);
            return lift_to_extended(as_view(ct_pb), &crt);
        };
        RingEls lhs_lifted = lift(lhs);
        RingEls rhs_lifted = lift(rhs);
        WideRingEls acc = ring.allocate_wide(3, lhs_lifted.rns_base);
        hom_mul_raw_acc(acc, 0, lhs_lifted.data.view(), rhs_lifted.data.view());
        RingEls prod = ring.reduce_wide(acc, Basis::CRTBasis);
        ring.crt_to_pb(prod);
        RingEls rescaled = rescale_to_base(std::move(prod), base_len, t);
        return relin(as_view(rescaled), rk, output_basis);
    }
    /// src/bfv.rs:783-841 (one key per automorphism, in the order of `gs`)
    std::vector<RingEls> bfv_hom_gal(const RingView& ct, const std::vector<uint64_t>& gs,
                                     const std::vector<const KeySwitchKey*>& gks) {
        ORACLE_ASSERT(ct.basis == Basis::CRTBasis && ct.count() == 2, "hom_gal operand");
        std::vector<RingEls> results;
        if (gs.empty()) return results;
        const Base& base = ct.rns_base;
        size_t base_len = base.size();
        RingEls c1 = ring.clone_els(ct.rows(1, 2));
        ring.crt_to_pb(c1);
        Digits digits = clip_digits(gks[0]->digits, base_len);
        RingEls parts = gadget_decompose(as_view(c1), digits);
        RingEls gal_parts = ring.allocate_in_basis(parts.count(), base, Basis::CRTBasis);
        RingEls gal_c0 = ring.allocate_in_basis(1, base, Basis::CRTBasis);
        for (size_t gi = 0; gi < gs.size(); gi++) {
            const KeySwitchKey& gk = *gks[gi];
            ORACLE_ASSERT(digits == clip_digits(gk.digits, base_len), "all galois keys must use the same digits");
            ring.apply_galois(gal_parts, as_view(parts), gs[gi]);
            ring.apply_galois(gal_c0, ct.rows(0, 1), gs[gi]);
            WideRingEls acc = ring.allocate_wide(2, base);
            std::vector<std::tuple<V64, u128, V64, u128>> terms;
            for (size_t i = 0; i < digits.size(); i++) {
                RingView key = as_view(gk.keys[i]).restrict_base(base_len);
                terms.emplace_back(gal_parts.data.view().rows(i, i + 1), gal_parts.bound, key.data, key.bound);
            }
            if (!terms.empty()) acc.inner_product(ring.backend, 0, 2, terms);
            acc.add(ring.backend, 0, 1, gal_c0.data.view(), gal_c0.bound);
            results.push_back(ring.reduce_wide(acc, Basis::CRTBasis));
        }
        return results;
    }
};

}  // namespace oracle
