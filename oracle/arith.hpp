// ORACLE — test infrastructure only. Nothing in the product library includes, links or runs
// this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
// checker. It restates the reference's scalar arithmetic line by line:
//   MontgomeryModulus    cyclosubfield-dbfv/src/hal/mont.rs:4-77
//   mul_mod / pow_mod    cyclosubfield-dbfv/src/hal/ntt.rs:87-100
//   find_root_of_unity   cyclosubfield-dbfv/src/hal/ntt.rs:104-115
//   rounded_div          cyclosubfield-dbfv/src/hal/ntt.rs:118-121
//   BarrettMul           cyclosubfield-dbfv/src/hal/ntt.rs:126-158
// Rust's wrapping arithmetic is written with unsigned casts, so no signed overflow (UB) occurs.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>

namespace oracle {

typedef __int128 i128;
typedef unsigned __int128 u128;

static const i128 I128_MAX = (i128)(~(u128)0 >> 1);
static const u128 I64_MAX_U = (u128)INT64_MAX;

inline int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
inline int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
inline int64_t wmul(int64_t a, int64_t b) { return (int64_t)((uint64_t)a * (uint64_t)b); }
inline i128 wadd128(i128 a, i128 b) { return (i128)((u128)a + (u128)b); }
inline i128 wsub128(i128 a, i128 b) { return (i128)((u128)a - (u128)b); }
inline i128 wmul128(i128 a, i128 b) { return (i128)((u128)a * (u128)b); }
inline i128 rem_euclid128(i128 a, i128 m) {
    i128 r = a % m;
    return r < 0 ? r + (m < 0 ? -m : m) : r;
}
inline int64_t rem_euclid64(int64_t a, int64_t m) {
    int64_t r = a % m;
    return r < 0 ? r + m : r;
}

[[noreturn]] inline void fail(const std::string& msg) { throw std::runtime_error(msg); }
#define ORACLE_ASSERT(cond, msg)                                                                   \
    do {                                                                                           \
        if (!(cond)) ::oracle::fail(std::string("oracle assertion failed: ") + (msg));            \
    } while (0)

// ---------------------------------------------------------------------------------------------
// src/hal/mont.rs
// ---------------------------------------------------------------------------------------------

/// Signed Montgomery arithmetic with R = 2^64 (src/hal/mont.rs:4-77).
struct MontgomeryModulus {
    int64_t N;
    int64_t neg_inv_N;
    int64_t R_sqr_mod_N;
    int64_t R_cbe_mod_N;

    /// src/hal/mont.rs:13-33. `-N^-1 mod 2^64` is unique, so it is computed here by Newton
    /// iteration instead of the extended Euclidean algorithm the reference uses; the low 64 bits
    /// agree. `pmod` returns values in (0, N].
    static MontgomeryModulus create(int64_t N) {
        ORACLE_ASSERT(N > 1 && (N & 1), "modulus must be odd and > 1");
        uint64_t inv = (uint64_t)N;
        for (int i = 0; i < 7; i++) inv *= 2 - (uint64_t)N * inv;
        auto pmod = [N](i128 x) -> int64_t {
            i128 res = (x % (i128)N) + (i128)N;
            if (res > (i128)N) res -= N;
            return (int64_t)res;
        };
        MontgomeryModulus m;
        m.N = N;
        m.neg_inv_N = (int64_t)(0 - inv);
        i128 R_mod_N = pmod((i128)1 << 64);
        m.R_sqr_mod_N = pmod(R_mod_N * R_mod_N);
        m.R_cbe_mod_N = pmod((i128)m.R_sqr_mod_N * (i128)pmod((i128)1 << 64));
        return m;
    }

    /// src/hal/mont.rs:41-45: |x| <= 2^63 N + N  ->  [-N, N], congruent to 2^-64 x.
    int64_t red128(i128 x) const {
        int64_t m = wmul((int64_t)x, neg_inv_N);
        i128 t = (i128)m * (i128)N;
        return (int64_t)(wadd128(x, t) >> 64);
    }

    /// src/hal/mont.rs:60-66: any i128 -> [-N, N], congruent to 2^-128 x.
    int64_t double_red128(i128 x) const {
        int64_t m = wmul((int64_t)x, neg_inv_N);
        i128 t = (i128)m * (i128)N;
        i128 carry = (i128)((((u128)(uint64_t)x) + ((u128)(uint64_t)t)) >> 64);
        i128 r1 = (x >> 64) + (t >> 64) + carry;
        return red128(r1);
    }

    /// src/hal/mont.rs:70
    int64_t to_mont64(int64_t x) const { return red128((i128)x * (i128)R_sqr_mod_N); }

    /// src/hal/mont.rs:74-76
    int64_t to_mont128(i128 x) const { return red128((i128)red128(x) * (i128)R_cbe_mod_N); }
};

// ---------------------------------------------------------------------------------------------
// src/hal/ntt.rs helpers
// ---------------------------------------------------------------------------------------------

/// src/hal/ntt.rs:87
inline int64_t mul_mod(int64_t a, int64_t b, int64_t q) { return (int64_t)(((i128)a * (i128)b) % (i128)q); }

/// src/hal/ntt.rs:89-100 (`b %= q` truncates, as Rust's `%`).
inline int64_t pow_mod(int64_t b, uint64_t e, int64_t q) {
    int64_t result = 1;
    b %= q;
    while (e > 0) {
        if (e & 1) result = mul_mod(result, b, q);
        b = mul_mod(b, b, q);
        e >>= 1;
    }
    return result;
}

inline bool is_power_of_two(uint64_t x) { return x != 0 && (x & (x - 1)) == 0; }

/// src/hal/ntt.rs:104-115
inline int64_t find_root_of_unity(int64_t q, uint64_t n) {
    ORACLE_ASSERT(n > 1, "root of unity order must be > 1");
    ORACLE_ASSERT((q - 1) % (int64_t)n == 0, "modulus doesn't support roots of unity of this order");
    uint64_t p = is_power_of_two(n) ? 2 : 3;
    for (int64_t candidate = 2;; candidate++) {
        int64_t root = pow_mod(candidate, (uint64_t)((q - 1) / (int64_t)n), q);
        if (pow_mod(root, n / p, q) != 1) return root;
    }
}

/// src/hal/ntt.rs:118-121: round(a / b) for b > 0, half away from zero.
inline i128 rounded_div(i128 a, i128 b) { return a >= 0 ? (a + b / 2) / b : -((-a + b / 2) / b); }

/// Barrett multiplication by a constant (src/hal/ntt.rs:126-158).
struct BarrettMul {
    int64_t z;
    int64_t u;

    static BarrettMul create(int64_t value, int64_t n) {
        ORACLE_ASSERT(n > 1 && n % 2 == 1 && n < ((int64_t)1 << 62), "bad Barrett modulus");
        int64_t z = value % n;
        if (2 * (i128)z > n) z -= n;
        else if (2 * (i128)z < -n) z += n;
        i128 u = rounded_div(-((i128)z << 64), (i128)n);
        ORACLE_ASSERT(u >= INT64_MIN && u <= INT64_MAX, "Barrett constant overflow");
        return BarrettMul{z, (int64_t)u};
    }

    /// src/hal/ntt.rs:149-152
    int64_t mul(int64_t x, int64_t n) const {
        int64_t q = (int64_t)(((i128)u * (i128)x + ((i128)1 << 63)) >> 64);
        return wadd(wmul(z, x), wmul(q, n));
    }

    bool is_one() const { return z == 1; }
};

}  // namespace oracle
