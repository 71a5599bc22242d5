/*
 * op_count.h -- an FP32 number type that counts its own arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  sms_oracle.cpp compiled with -DORC_OPCOUNT uses
 * CFloat as its scalar type (liboracle_ops.so).  Every value is still an IEEE
 * float computed in the same order as the plain oracle build, so results are
 * bit-identical to liboracle.so; each operation also increments a per-thread
 * counter.  The counts are the algorithmic FP32 work of a walk: what the
 * measurement's FLOP/s figures divide by kernel time.
 *
 * Counting rules: add, sub, mul, div and sqrt count 1 each (a fused
 * multiply-add on the GPU is the mul and the add it replaces, 2 FLOPs);
 * transcendentals (acos, asin, atan2, sin, cos, tan, exp, log, log2, erf)
 * count 1 each and are also counted separately.  Comparisons, min/max, abs,
 * copysign, floor/ceil, negation and conversions are not counted.
 */
#pragma once

#include <cmath>
#include <atomic>
#include <cstdint>
#include <type_traits>

namespace orc_opcount {

/* add .. transc: every counted operation.  box, tri: BVH box tests and
 * ray-triangle tests; box_flops, tri_flops: the FLOPs inside those tests (a
 * subset of the first five), so that traversal work can be scaled by the GPU's
 * own node and triangle counts, which depend on its tree; rays: scene ray
 * casts (closest hit and occlusion). */
struct Counters {
    uint64_t add = 0, mul = 0, div = 0, sqrt = 0, transc = 0;
    uint64_t box = 0, tri = 0, box_flops = 0, tri_flops = 0, rays = 0;
    uint64_t flops() const { return add + mul + div + sqrt + transc; }
};
const int kNumCounters = 10;

/* Totals of the threads that have exited (worker threads of a batch call). */
inline std::atomic<uint64_t> *totals() {
    static std::atomic<uint64_t> t[kNumCounters];
    return t;
}

/* Per-thread counters; a worker adds its counts to totals() when it exits,
 * so after a batch call has joined its workers totals() + the calling
 * thread's own counters hold everything the call did. */
struct ThreadCounters {
    Counters c;
    ~ThreadCounters() {
        std::atomic<uint64_t> *t = totals();
        t[0] += c.add; t[1] += c.mul; t[2] += c.div; t[3] += c.sqrt; t[4] += c.transc;
        t[5] += c.box; t[6] += c.tri; t[7] += c.box_flops; t[8] += c.tri_flops; t[9] += c.rays;
    }
};

inline Counters &counters() {
    static thread_local ThreadCounters tc;
    return tc.c;
}

inline void read_counters(uint64_t out[kNumCounters]) {
    const Counters &c = counters();
    std::atomic<uint64_t> *t = totals();
    out[0] = t[0] + c.add; out[1] = t[1] + c.mul; out[2] = t[2] + c.div;
    out[3] = t[3] + c.sqrt; out[4] = t[4] + c.transc;
    out[5] = t[5] + c.box; out[6] = t[6] + c.tri; out[7] = t[7] + c.box_flops; out[8] = t[8] + c.tri_flops;
    out[9] = t[9] + c.rays;
}

inline void reset_counters() {
    counters() = Counters();
    for (int i = 0; i < kNumCounters; ++i) totals()[i] = 0;
}

/* Counts one box (is_tri false) or triangle test and the FLOPs spent inside it. */
struct TraversalScope {
    bool tri;
    uint64_t start;
    explicit TraversalScope(bool is_tri) : tri(is_tri), start(counters().flops()) {}
    ~TraversalScope() {
        Counters &c = counters();
        if (tri) { ++c.tri; c.tri_flops += c.flops() - start; }
        else { ++c.box; c.box_flops += c.flops() - start; }
    }
};

struct CFloat {
    float v = 0.f;
    CFloat() {}
    template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>
    CFloat(T x) : v((float)x) {}
    /* implicit to float (stores into the caller's float buffers), explicit to
     * everything else */
    operator float() const { return v; }
    template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value && !std::is_same<T, float>::value>>
    explicit operator T() const { return (T)v; }
    CFloat operator-() const { CFloat r; r.v = -v; return r; }
    CFloat &operator+=(CFloat b) { ++counters().add; v += b.v; return *this; }
    CFloat &operator-=(CFloat b) { ++counters().add; v -= b.v; return *this; }
    CFloat &operator*=(CFloat b) { ++counters().mul; v *= b.v; return *this; }
    CFloat &operator/=(CFloat b) { ++counters().div; v /= b.v; return *this; }
};

inline CFloat mk(float x) { CFloat r; r.v = x; return r; }
inline float val(CFloat a) { return a.v; }
template <class T, class = std::enable_if_t<std::is_arithmetic<T>::value>>
inline float val(T a) { return (float)a; }

/* Operands a counted operation accepts beside CFloat: float and integers.  A
 * double operand takes the built-in operator instead (CFloat converts to float,
 * then to double), which computes in double exactly as the float build does. */
template <class T>
using is_operand = std::integral_constant<bool, std::is_same<T, CFloat>::value || std::is_same<T, float>::value ||
                                                    std::is_integral<T>::value>;
template <class A, class B>
using both = std::enable_if_t<(std::is_same<A, CFloat>::value || std::is_same<B, CFloat>::value) &&
                              is_operand<A>::value && is_operand<B>::value>;

template <class A, class B, class = both<A, B>>
inline CFloat operator+(A a, B b) { ++counters().add; return mk(val(a) + val(b)); }
template <class A, class B, class = both<A, B>>
inline CFloat operator-(A a, B b) { ++counters().add; return mk(val(a) - val(b)); }
template <class A, class B, class = both<A, B>>
inline CFloat operator*(A a, B b) { ++counters().mul; return mk(val(a) * val(b)); }
template <class A, class B, class = both<A, B>>
inline CFloat operator/(A a, B b) { ++counters().div; return mk(val(a) / val(b)); }
template <class A, class B, class = both<A, B>>
inline bool operator<(A a, B b) { return val(a) < val(b); }
template <class A, class B, class = both<A, B>>
inline bool operator>(A a, B b) { return val(a) > val(b); }
template <class A, class B, class = both<A, B>>
inline bool operator<=(A a, B b) { return val(a) <= val(b); }
template <class A, class B, class = both<A, B>>
inline bool operator>=(A a, B b) { return val(a) >= val(b); }
template <class A, class B, class = both<A, B>>
inline bool operator==(A a, B b) { return val(a) == val(b); }
template <class A, class B, class = both<A, B>>
inline bool operator!=(A a, B b) { return val(a) != val(b); }

inline CFloat counted_sqrt(CFloat a) { ++counters().sqrt; return mk(std::sqrt(a.v)); }
inline CFloat counted_transc(float r) { ++counters().transc; return mk(r); }

} // namespace orc_opcount

/* Overloads of the <cmath> functions the oracle calls with std:: qualification.
 * The float overloads they forward to are the ones the plain build calls. */
namespace std {
using orc_opcount::CFloat;
template <> struct common_type<CFloat, CFloat> { typedef CFloat type; };
template <class T> struct common_type<CFloat, T> { typedef CFloat type; };
template <class T> struct common_type<T, CFloat> { typedef CFloat type; };
inline CFloat sqrt(CFloat a) { return orc_opcount::counted_sqrt(a); }
inline CFloat fabs(CFloat a) { return orc_opcount::mk(std::fabs(a.v)); }
inline CFloat floor(CFloat a) { return orc_opcount::mk(std::floor(a.v)); }
inline CFloat ceil(CFloat a) { return orc_opcount::mk(std::ceil(a.v)); }
inline bool isnan(CFloat a) { return std::isnan(a.v); }
inline bool isfinite(CFloat a) { return std::isfinite(a.v); }
template <class B>
inline CFloat copysign(CFloat a, B b) { return orc_opcount::mk(std::copysign(a.v, orc_opcount::val(b))); }
inline CFloat copysign(float a, CFloat b) { return orc_opcount::mk(std::copysign(a, b.v)); }
inline CFloat acos(CFloat a) { return orc_opcount::counted_transc(std::acos(a.v)); }
inline CFloat asin(CFloat a) { return orc_opcount::counted_transc(std::asin(a.v)); }
inline CFloat sin(CFloat a) { return orc_opcount::counted_transc(std::sin(a.v)); }
inline CFloat cos(CFloat a) { return orc_opcount::counted_transc(std::cos(a.v)); }
inline CFloat tan(CFloat a) { return orc_opcount::counted_transc(std::tan(a.v)); }
inline CFloat exp(CFloat a) { return orc_opcount::counted_transc(std::exp(a.v)); }
inline CFloat log(CFloat a) { return orc_opcount::counted_transc(std::log(a.v)); }
inline CFloat log2(CFloat a) { return orc_opcount::counted_transc(std::log2(a.v)); }
inline CFloat erf(CFloat a) { return orc_opcount::counted_transc(std::erf(a.v)); }
template <class B>
inline CFloat atan2(CFloat a, B b) { return orc_opcount::counted_transc(std::atan2(a.v, orc_opcount::val(b))); }
inline CFloat atan2(float a, CFloat b) { return orc_opcount::counted_transc(std::atan2(a, b.v)); }
} // namespace std
