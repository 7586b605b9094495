// wgsl_rt.h — C++ runtime for compute shaders translated from WGSL by wgsl_ref.py.
//
// Test infrastructure only: the translated shader is a second, mechanical oracle
// for the raycast pass, built from the reference's own shader source. Nothing in
// the product includes this file.
//
// Values: WGSL scalars are float / uint32_t / int32_t / bool; vecN<T> is Vec<T, N>;
// array<T, N> is std::array. Arithmetic is IEEE binary32 with one rounding per
// operation (compile with -ffp-contract=off -fno-fast-math).
//
// Where WGSL leaves a result to the implementation, this runtime pins it to the
// same choice as the C oracle (woxel_oracle.c) and the CUDA kernels:
//   min / max      a NaN operand yields the other operand; otherwise the usual order
//                  comparison (min(+0, -0) returns the first operand);
//   normalize(v)   v / sqrt(dot(v, v)), each component divided, correctly rounded;
//   dot(a, b)      ((a.x*b.x + a.y*b.y) + a.z*b.z) [+ a.w*b.w];
//   mix(a, b, t)   a * (1 - t) + b * t;
//   f32 -> i32/u32 truncation toward zero, saturating, NaN -> 0;
//   x % y (f32)    x - y * trunc(x / y), as the WGSL specification writes it;
//   rgba8unorm     NaN and x <= 0 -> 0, x >= 1 -> 255, else floor(x * 255 + 0.5).
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <type_traits>

namespace wgsl {

template <class T, int N>
struct Vec {
    T c[N];
    T &operator[](uint32_t i) { return c[i]; }
    const T &operator[](uint32_t i) const { return c[i]; }
};

template <class T>
struct is_vec : std::false_type {};
template <class T, int N>
struct is_vec<Vec<T, N>> : std::true_type {};

// ---------------------------------------------------------------- conversions
template <class To, class From>
inline To cvt_scalar(From x) {
    if constexpr (std::is_same_v<To, From>) {
        return x;
    } else if constexpr (std::is_same_v<To, bool>) {
        return x != From(0);
    } else if constexpr (std::is_same_v<From, bool>) {
        return x ? To(1) : To(0);
    } else if constexpr (std::is_floating_point_v<From> && std::is_integral_v<To>) {
        if (x != x) return To(0);
        const float lo = std::is_signed_v<To> ? -2147483648.0f : 0.0f;
        const float hi = std::is_signed_v<To> ? 2147483648.0f : 4294967296.0f;
        if (x <= lo) return std::is_signed_v<To> ? To(INT32_MIN) : To(0);
        if (x >= hi) return std::is_signed_v<To> ? To(INT32_MAX) : To(UINT32_MAX);
        return static_cast<To>(x);
    } else {
        return static_cast<To>(x);  // integer <-> integer (two's complement), integer -> f32 (nearest)
    }
}

template <class To, class From>
inline auto cvt(const From &x) {
    if constexpr (is_vec<From>::value) {
        constexpr int N = sizeof(From) / sizeof(x.c[0]);
        Vec<To, N> r;
        for (int i = 0; i < N; i++) r.c[i] = cvt_scalar<To>(x.c[i]);
        return r;
    } else {
        return cvt_scalar<To>(x);
    }
}

// Number of scalar components of a constructor argument.
template <class A>
constexpr int ncomp() {
    if constexpr (is_vec<A>::value) return sizeof(A) / sizeof(std::declval<A>().c[0]);
    else return 1;
}
template <class T, int N, class A>
inline void put(Vec<T, N> &r, int &k, const A &a) {
    if constexpr (is_vec<A>::value) {
        for (int i = 0; i < ncomp<A>(); i++) r.c[k++] = cvt_scalar<T>(a.c[i]);
    } else {
        r.c[k++] = cvt_scalar<T>(a);
    }
}

// vecN<T>(...): zero, splat of one scalar, conversion of one vector, or components.
template <class T, int N, class... A>
inline Vec<T, N> vec(const A &...a) {
    Vec<T, N> r{};
    if constexpr (sizeof...(A) == 0) {
        return r;
    } else if constexpr (sizeof...(A) == 1 && (!is_vec<A>::value && ...)) {
        for (int i = 0; i < N; i++) r.c[i] = cvt_scalar<T>(a...);
        return r;
    } else {
        static_assert((ncomp<A>() + ...) == N, "vector constructor: wrong number of components");
        int k = 0;
        (put(r, k, a), ...);
        return r;
    }
}

template <class A>
struct elem { using type = A; };
template <class T, int N>
struct elem<Vec<T, N>> { using type = T; };

// vecN(...) without a component type: the type of the arguments' components
// (f32 if any is f32, else u32, else i32, else bool).
template <class... A>
struct auto_elem {
    static constexpr bool f = (std::is_floating_point_v<typename elem<A>::type> || ...);
    static constexpr bool u = (std::is_same_v<typename elem<A>::type, uint32_t> || ...);
    static constexpr bool b = (std::is_same_v<typename elem<A>::type, bool> && ...);
    using type = std::conditional_t<f, float, std::conditional_t<u, uint32_t, std::conditional_t<b, bool, int32_t>>>;
};
template <int N, class... A>
inline auto vec_auto(const A &...a) {
    return vec<typename auto_elem<A...>::type, N>(a...);
}

// ---------------------------------------------------------------- swizzles
template <int... I, class T, int N>
inline Vec<T, (int)sizeof...(I)> swz(const Vec<T, N> &v) {
    return Vec<T, (int)sizeof...(I)>{{v.c[I]...}};
}

// ---------------------------------------------------------------- operators
template <class T>
inline T bin_arith(char op, T a, T b) {
    switch (op) {
        case '+': return a + b;
        case '-': return a - b;
        case '*': return a * b;
        default:
            if constexpr (std::is_integral_v<T>) {
                if (b == T(0)) return a;  // WGSL: integer division by zero yields e1
                if constexpr (std::is_signed_v<T>)
                    if (a == INT32_MIN && b == T(-1)) return a;
            }
            return a / b;
    }
}

#define WGSL_VEC_ARITH(OP, CH)                                                          \
    template <class T, int N>                                                           \
    inline Vec<T, N> operator OP(const Vec<T, N> &a, const Vec<T, N> &b) {               \
        Vec<T, N> r;                                                                    \
        for (int i = 0; i < N; i++) r.c[i] = bin_arith<T>(CH, a.c[i], b.c[i]);          \
        return r;                                                                       \
    }                                                                                   \
    template <class T, int N, class S, std::enable_if_t<!is_vec<S>::value, int> = 0>    \
    inline Vec<T, N> operator OP(const Vec<T, N> &a, S s) {                             \
        Vec<T, N> r;                                                                    \
        for (int i = 0; i < N; i++) r.c[i] = bin_arith<T>(CH, a.c[i], static_cast<T>(s)); \
        return r;                                                                       \
    }                                                                                   \
    template <class T, int N, class S, std::enable_if_t<!is_vec<S>::value, int> = 0>    \
    inline Vec<T, N> operator OP(S s, const Vec<T, N> &a) {                             \
        Vec<T, N> r;                                                                    \
        for (int i = 0; i < N; i++) r.c[i] = bin_arith<T>(CH, static_cast<T>(s), a.c[i]); \
        return r;                                                                       \
    }                                                                                   \
    template <class T, int N, class B>                                                  \
    inline Vec<T, N> &operator OP##=(Vec<T, N> &a, const B &b) {                        \
        a = a OP b;                                                                     \
        return a;                                                                       \
    }
WGSL_VEC_ARITH(+, '+')
WGSL_VEC_ARITH(-, '-')
WGSL_VEC_ARITH(*, '*')
WGSL_VEC_ARITH(/, '/')
#undef WGSL_VEC_ARITH

template <class T, int N>
inline Vec<T, N> operator-(const Vec<T, N> &a) {
    Vec<T, N> r;
    for (int i = 0; i < N; i++) r.c[i] = -a.c[i];
    return r;
}
template <int N>
inline Vec<bool, N> operator!(const Vec<bool, N> &a) {
    Vec<bool, N> r;
    for (int i = 0; i < N; i++) r.c[i] = !a.c[i];
    return r;
}

// Comparisons give vectors of bool; a scalar operand is splatted.
#define WGSL_VEC_CMP(OP)                                                               \
    template <class T, int N>                                                          \
    inline Vec<bool, N> operator OP(const Vec<T, N> &a, const Vec<T, N> &b) {           \
        Vec<bool, N> r;                                                                \
        for (int i = 0; i < N; i++) r.c[i] = a.c[i] OP b.c[i];                         \
        return r;                                                                      \
    }                                                                                  \
    template <class T, int N, class S, std::enable_if_t<!is_vec<S>::value, int> = 0>   \
    inline Vec<bool, N> operator OP(const Vec<T, N> &a, S s) {                         \
        Vec<bool, N> r;                                                                \
        for (int i = 0; i < N; i++) r.c[i] = a.c[i] OP static_cast<T>(s);              \
        return r;                                                                      \
    }                                                                                  \
    template <class T, int N, class S, std::enable_if_t<!is_vec<S>::value, int> = 0>   \
    inline Vec<bool, N> operator OP(S s, const Vec<T, N> &a) {                         \
        Vec<bool, N> r;                                                                \
        for (int i = 0; i < N; i++) r.c[i] = static_cast<T>(s) OP a.c[i];              \
        return r;                                                                      \
    }
WGSL_VEC_CMP(==)
WGSL_VEC_CMP(!=)
WGSL_VEC_CMP(<)
WGSL_VEC_CMP(<=)
WGSL_VEC_CMP(>)
WGSL_VEC_CMP(>=)
#undef WGSL_VEC_CMP

// Bitwise &, |, ^ (also on bool and vectors of bool) and shifts; the result has the
// left operand's type.
template <class A, class B>
inline auto bitop(char op, const A &a, const B &b) {
    if constexpr (is_vec<A>::value || is_vec<B>::value) {
        using V = std::conditional_t<is_vec<A>::value, A, B>;
        using T = typename elem<V>::type;
        V r;
        for (int i = 0; i < ncomp<V>(); i++) {
            T x, y;
            if constexpr (is_vec<A>::value) x = a.c[i]; else x = static_cast<T>(a);
            if constexpr (is_vec<B>::value) y = b.c[i]; else y = static_cast<T>(b);
            r.c[i] = bitop(op, x, y);
        }
        return r;
    } else {
        const A y = static_cast<A>(b);
        switch (op) {
            case '&': return static_cast<A>(a & y);
            case '|': return static_cast<A>(a | y);
            default: return static_cast<A>(a ^ y);
        }
    }
}
template <class A, class B>
inline auto band(const A &a, const B &b) { return bitop('&', a, b); }
template <class A, class B>
inline auto bor(const A &a, const B &b) { return bitop('|', a, b); }
template <class A, class B>
inline auto bxor(const A &a, const B &b) { return bitop('^', a, b); }

template <class T>
inline T shl_s(T a, uint32_t n) { return static_cast<T>(static_cast<std::make_unsigned_t<T>>(a) << (n & 31u)); }
template <class T>
inline T shr_s(T a, uint32_t n) { return static_cast<T>(a >> (n & 31u)); }  // arithmetic for i32
template <class A, class B>
inline A shl(const A &a, const B &b) {
    if constexpr (is_vec<A>::value) {
        A r;
        for (int i = 0; i < ncomp<A>(); i++) {
            uint32_t n;
            if constexpr (is_vec<B>::value) n = static_cast<uint32_t>(b.c[i]); else n = static_cast<uint32_t>(b);
            r.c[i] = shl_s(a.c[i], n);
        }
        return r;
    } else {
        return shl_s(a, static_cast<uint32_t>(b));
    }
}
template <class A, class B>
inline A shr(const A &a, const B &b) {
    if constexpr (is_vec<A>::value) {
        A r;
        for (int i = 0; i < ncomp<A>(); i++) {
            uint32_t n;
            if constexpr (is_vec<B>::value) n = static_cast<uint32_t>(b.c[i]); else n = static_cast<uint32_t>(b);
            r.c[i] = shr_s(a.c[i], n);
        }
        return r;
    } else {
        return shr_s(a, static_cast<uint32_t>(b));
    }
}

// x % y: integers truncate (e1 for a zero divisor); f32 as x - y * trunc(x / y).
template <class T>
inline T mod_s(T a, T b) {
    if constexpr (std::is_floating_point_v<T>) {
        return a - b * std::trunc(a / b);
    } else {
        if (b == T(0)) return a;
        if constexpr (std::is_signed_v<T>)
            if (a == INT32_MIN && b == T(-1)) return T(0);
        return a % b;
    }
}
template <class A, class B>
inline auto mod(const A &a, const B &b) {
    if constexpr (is_vec<A>::value || is_vec<B>::value) {
        using V = std::conditional_t<is_vec<A>::value, A, B>;
        using T = typename elem<V>::type;
        V r;
        for (int i = 0; i < ncomp<V>(); i++) {
            T x, y;
            if constexpr (is_vec<A>::value) x = a.c[i]; else x = static_cast<T>(a);
            if constexpr (is_vec<B>::value) y = b.c[i]; else y = static_cast<T>(b);
            r.c[i] = mod_s(x, y);
        }
        return r;
    } else {
        return mod_s(a, static_cast<A>(b));
    }
}

// ---------------------------------------------------------------- built-ins
template <class F, class A>
inline A map1(F f, const A &a) {
    if constexpr (is_vec<A>::value) {
        A r;
        for (int i = 0; i < ncomp<A>(); i++) r.c[i] = f(a.c[i]);
        return r;
    } else {
        return f(a);
    }
}
template <class F, class A, class B>
inline auto map2(F f, const A &a, const B &b) {
    if constexpr (is_vec<A>::value || is_vec<B>::value) {
        using V = std::conditional_t<is_vec<A>::value, A, B>;
        using T = typename elem<V>::type;
        V r;
        for (int i = 0; i < ncomp<V>(); i++) {
            T x, y;
            if constexpr (is_vec<A>::value) x = a.c[i]; else x = static_cast<T>(a);
            if constexpr (is_vec<B>::value) y = b.c[i]; else y = static_cast<T>(b);
            r.c[i] = f(x, y);
        }
        return r;
    } else {
        return f(a, static_cast<A>(b));
    }
}

template <class T>
inline T min_s(T a, T b) {
    if constexpr (std::is_floating_point_v<T>) {
        if (a != a) return b;
        if (b != b) return a;
    }
    return (b < a) ? b : a;
}
template <class T>
inline T max_s(T a, T b) {
    if constexpr (std::is_floating_point_v<T>) {
        if (a != a) return b;
        if (b != b) return a;
    }
    return (b > a) ? b : a;
}
template <class A, class B>
inline auto min(const A &a, const B &b) {
    return map2([](auto x, auto y) { return min_s(x, y); }, a, b);
}
template <class A, class B>
inline auto max(const A &a, const B &b) {
    return map2([](auto x, auto y) { return max_s(x, y); }, a, b);
}
template <class A>
inline A floor(const A &a) { return map1([](auto x) { return std::floor(x); }, a); }
template <class A>
inline A trunc(const A &a) { return map1([](auto x) { return std::trunc(x); }, a); }
template <class A>
inline A abs(const A &a) {
    return map1([](auto x) {
        if constexpr (std::is_floating_point_v<decltype(x)>) return std::fabs(x);
        else if constexpr (std::is_signed_v<decltype(x)>) return x == INT32_MIN ? x : (x < 0 ? -x : x);
        else return x;
    }, a);
}
template <class A>
inline A sqrt(const A &a) { return map1([](auto x) { return std::sqrt(x); }, a); }

template <class T, int N>
inline T dot(const Vec<T, N> &a, const Vec<T, N> &b) {
    T s = a.c[0] * b.c[0];
    for (int i = 1; i < N; i++) s = s + a.c[i] * b.c[i];
    return s;
}
template <class T, int N>
inline T length(const Vec<T, N> &a) { return std::sqrt(dot(a, a)); }
template <class T, int N>
inline Vec<T, N> normalize(const Vec<T, N> &a) {
    const T l = std::sqrt(dot(a, a));
    Vec<T, N> r;
    for (int i = 0; i < N; i++) r.c[i] = a.c[i] / l;
    return r;
}
template <class A, class B, class C>
inline A mix(const A &a, const B &b, const C &t) {
    if constexpr (is_vec<A>::value) {
        A r;
        for (int i = 0; i < ncomp<A>(); i++) {
            float ti;
            if constexpr (is_vec<C>::value) ti = t.c[i]; else ti = t;
            const float omt = 1.0f - ti;
            r.c[i] = a.c[i] * omt + b.c[i] * ti;
        }
        return r;
    } else {
        const float omt = 1.0f - t;
        return a * omt + b * t;
    }
}
template <class A, class B, class C>
inline A select(const A &f, const B &t, const C &cond) {
    if constexpr (is_vec<C>::value) {
        A r;
        for (int i = 0; i < ncomp<A>(); i++) r.c[i] = cond.c[i] ? t.c[i] : f.c[i];
        return r;
    } else {
        return cond ? static_cast<A>(t) : f;
    }
}
template <int N>
inline bool all(const Vec<bool, N> &a) {
    for (int i = 0; i < N; i++)
        if (!a.c[i]) return false;
    return true;
}
template <int N>
inline bool any(const Vec<bool, N> &a) {
    for (int i = 0; i < N; i++)
        if (a.c[i]) return true;
    return false;
}
inline bool all(bool a) { return a; }
inline bool any(bool a) { return a; }

// ---------------------------------------------------------------- resources
// texture_3d<T>: texel (x, y, z) at (z * H + y) * W + x; out-of-range loads give 0.
template <class T>
struct Tex3 {
    const T *data = nullptr;
    uint32_t w = 0, h = 0, d = 0;
};
template <class T, class C>
inline Vec<T, 4> textureLoad(const Tex3<T> &t, const C &coord, int32_t /*level*/) {
    const uint32_t x = static_cast<uint32_t>(coord.c[0]), y = static_cast<uint32_t>(coord.c[1]),
                   z = static_cast<uint32_t>(coord.c[2]);
    Vec<T, 4> r{};
    r.c[3] = T(1);
    if (x < t.w && y < t.h && z < t.d) r.c[0] = t.data[(static_cast<uint64_t>(z) * t.h + y) * t.w + x];
    return r;
}
template <class T>
inline Vec<uint32_t, 3> textureDimensions(const Tex3<T> &t) {
    return Vec<uint32_t, 3>{{t.w, t.h, t.d}};
}

// texture_storage_2d<rgba8unorm, write>: 4 bytes per texel, row-major.
struct TexStore2 {
    uint8_t *data = nullptr;
    uint32_t w = 0, h = 0;
};
inline uint8_t unorm8(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 1.0f) return 255;
    return static_cast<uint8_t>(std::floor(x * 255.0f + 0.5f));
}
template <class C>
inline void textureStore(TexStore2 &t, const C &coord, const Vec<float, 4> &v) {
    const uint32_t x = static_cast<uint32_t>(coord.c[0]), y = static_cast<uint32_t>(coord.c[1]);
    if (x >= t.w || y >= t.h) return;
    uint8_t *p = t.data + 4 * (static_cast<uint64_t>(y) * t.w + x);
    for (int i = 0; i < 4; i++) p[i] = unorm8(v.c[i]);
}

// Runtime-sized storage array: element i at base + i * stride (the WGSL layout),
// loaded by the translator's generated loader; out-of-range reads give a zero element.
template <class E>
struct Storage {
    const uint8_t *base = nullptr;
    uint64_t stride = 0;
    uint32_t count = 0;
    E (*load)(const uint8_t *) = nullptr;
    E operator[](uint32_t i) const {
        if (i >= count) return E{};
        return load(base + static_cast<uint64_t>(i) * stride);
    }
};
template <class E>
inline uint32_t arrayLength(const Storage<E> &s) { return s.count; }

template <class T>
inline T load_scalar(const uint8_t *p) {
    T v;
    std::memcpy(&v, p, sizeof(T));
    return v;
}
// array<T, N> of 4-byte scalars stored without padding.
template <class T, size_t N>
inline std::array<T, N> load_array(const uint8_t *p) {
    std::array<T, N> v;
    std::memcpy(v.data(), p, sizeof(T) * N);
    return v;
}

}  // namespace wgsl
