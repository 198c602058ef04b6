// tg_common.cuh -- value types, complex arithmetic and error plumbing shared by
// the forward-path kernels.
//
// Value types: double, float (real systems) and cpx<double>, cpx<float>
// (complex systems, interleaved re/im, 16- or 8-byte aligned).  Block vectors
// are node-major: X[i * ld + c] is node i of right-hand side c, so one CSR
// entry a_ij multiplies a contiguous run of ld values of row j.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>
#include <cstdio>
#include <string>

namespace tg {

template <class R>
struct alignas(2 * sizeof(R)) cpx {
    R x, y;
};

using cd = cpx<double>;
using cf = cpx<float>;

template <class V> struct vt;
template <> struct vt<double> { using R = double; static constexpr bool cplx = false; };
template <> struct vt<float>  { using R = float;  static constexpr bool cplx = false; };
template <> struct vt<cd>     { using R = double; static constexpr bool cplx = true; };
template <> struct vt<cf>     { using R = float;  static constexpr bool cplx = true; };

#define TGHD __host__ __device__ __forceinline__

TGHD double re(double a) { return a; }
TGHD float re(float a) { return a; }
TGHD double re(cd a) { return a.x; }
TGHD float re(cf a) { return a.x; }
TGHD double im(double) { return 0.0; }
TGHD float im(float) { return 0.0f; }
TGHD double im(cd a) { return a.y; }
TGHD float im(cf a) { return a.y; }

template <class V> TGHD V vzero() { V v; memset(&v, 0, sizeof(V)); return v; }
template <> TGHD double vzero<double>() { return 0.0; }
template <> TGHD float vzero<float>() { return 0.0f; }
template <> TGHD cd vzero<cd>() { return cd{0.0, 0.0}; }
template <> TGHD cf vzero<cf>() { return cf{0.0f, 0.0f}; }

template <class R> TGHD cpx<R> operator+(cpx<R> a, cpx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <class R> TGHD cpx<R> operator-(cpx<R> a, cpx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> TGHD cpx<R> operator*(cpx<R> a, cpx<R> b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <class R> TGHD cpx<R> operator*(cpx<R> a, R s) { return {a.x * s, a.y * s}; }
template <class R> TGHD cpx<R>& operator+=(cpx<R>& a, cpx<R> b) { a.x += b.x; a.y += b.y; return a; }
template <class R> TGHD cpx<R>& operator-=(cpx<R>& a, cpx<R> b) { a.x -= b.x; a.y -= b.y; return a; }

// a*b for mixed real/complex scalar (complex: explicit fused multiply-adds,
// so kernels round alike)
TGHD double vmul(double a, double b) { return a * b; }
TGHD float vmul(float a, float b) { return a * b; }
TGHD cd vmul(cd a, cd b) { return {fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x)}; }
TGHD cf vmul(cf a, cf b) { return {fmaf(a.x, b.x, -(a.y * b.y)), fmaf(a.x, b.y, a.y * b.x)}; }
// acc - a*b (the forward/back substitution and residual kernels) and
// acc + a*b.  The complex forms are written as explicit chains of fused
// multiply-adds, so every kernel that uses them rounds alike whatever the
// compiler would contract.
TGHD double vfms(double acc, double a, double b) { return fma(-a, b, acc); }
TGHD float vfms(float acc, float a, float b) { return fmaf(-a, b, acc); }
TGHD cd vfms(cd acc, cd a, cd b) { return {fma(a.y, b.y, fma(-a.x, b.x, acc.x)), fma(-a.y, b.x, fma(-a.x, b.y, acc.y))}; }
TGHD cf vfms(cf acc, cf a, cf b) { return {fmaf(a.y, b.y, fmaf(-a.x, b.x, acc.x)), fmaf(-a.y, b.x, fmaf(-a.x, b.y, acc.y))}; }
TGHD double vfma(double acc, double a, double b) { return fma(a, b, acc); }
TGHD float vfma(float acc, float a, float b) { return fmaf(a, b, acc); }
TGHD cd vfma(cd acc, cd a, cd b) { return {fma(-a.y, b.y, fma(a.x, b.x, acc.x)), fma(a.y, b.x, fma(a.x, b.y, acc.y))}; }
TGHD cf vfma(cf acc, cf a, cf b) { return {fmaf(-a.y, b.y, fmaf(a.x, b.x, acc.x)), fmaf(a.y, b.x, fmaf(a.x, b.y, acc.y))}; }
// scale by a real scalar
TGHD double vscale(double a, double s) { return a * s; }
TGHD float vscale(float a, float s) { return a * s; }
TGHD cd vscale(cd a, double s) { return a * s; }
TGHD cf vscale(cf a, float s) { return a * s; }
TGHD double vadd(double a, double b) { return a + b; }
TGHD float vadd(float a, float b) { return a + b; }
TGHD cd vadd(cd a, cd b) { return a + b; }
TGHD cf vadd(cf a, cf b) { return a + b; }
TGHD double vsub(double a, double b) { return a - b; }
TGHD float vsub(float a, float b) { return a - b; }
TGHD cd vsub(cd a, cd b) { return a - b; }
TGHD cf vsub(cf a, cf b) { return a - b; }

// Re(conj(a) b): the real scalar products of the reference's complex
// BiCGSTAB (src/libmath/matrix_imp.hpp:364-391); the plain product for reals.
TGHD double redot(double a, double b) { return a * b; }
TGHD float redot(float a, float b) { return a * b; }
TGHD double redot(cd a, cd b) { return a.x * b.x + a.y * b.y; }
TGHD float redot(cf a, cf b) { return a.x * b.x + a.y * b.y; }
TGHD double nrm2(double a) { return a * a; }
TGHD float nrm2(float a) { return a * a; }
TGHD double nrm2(cd a) { return a.x * a.x + a.y * a.y; }
TGHD float nrm2(cf a) { return a.x * a.x + a.y * a.y; }
// The magnitude the componentwise backward-error test works with:
// max(|Re a|, |Im a|) as a float (within a factor sqrt 2 of |a|), formed
// from the bit pattern with integer operations (mantissa truncated to 23
// bits; below the FP32 range 0, above it inf), so the test costs no FP64
// arithmetic on a GPU whose FP64 rate is low.
TGHD float mag_bits(unsigned long long b)  // b: |x| as the bits of a double
{
    const int e = (int)(b >> 52) - 1023 + 127;
    if (e <= 0) return 0.0f;
    if (e >= 255) return __builtin_huge_valf();
    unsigned u = ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu);
    float f;
    memcpy(&f, &u, 4);
    return f;
}
TGHD unsigned long long abs_bits(double a)
{
    unsigned long long b;
    memcpy(&b, &a, 8);
    return b & 0x7fffffffffffffffull;
}
TGHD float mag1f(double a) { return mag_bits(abs_bits(a)); }
TGHD float mag1f(cd a)
{
    const unsigned long long x = abs_bits(a.x), y = abs_bits(a.y);  // non-negative: ordered as integers
    return mag_bits(x > y ? x : y);
}

// value conversion between precisions
template <class To, class From> TGHD To vcast(From a);
template <> TGHD double vcast<double, double>(double a) { return a; }
template <> TGHD float vcast<float, double>(double a) { return (float)a; }
template <> TGHD double vcast<double, float>(float a) { return (double)a; }
template <> TGHD float vcast<float, float>(float a) { return a; }
template <> TGHD cd vcast<cd, cd>(cd a) { return a; }
template <> TGHD cf vcast<cf, cd>(cd a) { return cf{(float)a.x, (float)a.y}; }
template <> TGHD cd vcast<cd, cf>(cf a) { return cd{(double)a.x, (double)a.y}; }
template <> TGHD cf vcast<cf, cf>(cf a) { return a; }

// complex square root, principal branch (same branch as std::sqrt)
TGHD cd csqrt_d(cd z)
{
    double r = hypot(z.x, z.y);
    if (r == 0.0) return cd{0.0, 0.0};
    if (z.x >= 0.0) {
        double t = sqrt(0.5 * (r + z.x));
        return cd{t, z.y / (2.0 * t)};
    }
    double t = sqrt(0.5 * (r - z.x));
    return cd{fabs(z.y) / (2.0 * t), z.y < 0.0 ? -t : t};
}

TGHD cd cdiv(cd a, cd b)
{
    // Smith's algorithm: scaled to avoid overflow
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, den = b.x + b.y * r;
        return cd{(a.x + a.y * r) / den, (a.y - a.x * r) / den};
    }
    double r = b.x / b.y, den = b.x * r + b.y;
    return cd{(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}

TGHD double vdiv(double a, double b) { return a / b; }
TGHD cd vdiv(cd a, cd b) { return cdiv(a, b); }
TGHD double vrecip(double a) { return 1.0 / a; }
TGHD cd vrecip(cd a) { return cdiv(cd{1.0, 0.0}, a); }

// ------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

struct Error {
    int code;
    std::string msg;
};

#define TG_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t _e = (call);                                                       \
        if (_e != cudaSuccess) {                                                       \
            throw ::tg::Error{3, std::string("CUDA error ") + cudaGetErrorString(_e) + \
                                     " at " + __FILE__ + ":" + std::to_string(__LINE__)}; \
        }                                                                              \
    } while (0)

#define TG_CHECK(cond, code, text)                     \
    do {                                               \
        if (!(cond)) throw ::tg::Error{code, (text)};  \
    } while (0)

constexpr int ROW_TILE = 32;  // rows per dot-partial tile (summation order fixed by it)

}  // namespace tg
