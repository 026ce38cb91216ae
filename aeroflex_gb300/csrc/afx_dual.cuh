// One-direction forward-mode dual number for the adjoint kernels.
//
// The face physics of afx_device.cuh is templated on its arithmetic type, so
// instantiating it with Dual gives the exact directional derivative of a face
// flux, ghost state or limiter value next to its value: one pass per input
// direction, all in registers.  The adjoint kernels use these columns of the
// local Jacobians on the fly and never store a Jacobian.
//
// Branches (entropy fix, limiter cases, characteristic boundary cases, min /
// max) follow the value, so the derivative is the one of the active branch.
#pragma once

#include <cuda_runtime.h>

namespace afx {
namespace dev {

struct Dual {
    double v, d;
    __device__ __forceinline__ Dual() : v(0), d(0) {}
    __device__ __forceinline__ Dual(double x) : v(x), d(0) {}
    __device__ __forceinline__ Dual(double x, double dx) : v(x), d(dx) {}
};

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double r = a.v / b.v;
    return Dual(r, (a.d - r * b.d) / b.v);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { return a = a * b; }
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(Dual a, Dual b) { return a.v >= b.v; }

__device__ __forceinline__ Dual dsqrt(Dual x) {
    const double s = sqrt(x.v);
    return Dual(s, x.d / (2.0 * s));
}
__device__ __forceinline__ Dual dabs(Dual x) { return x.v < 0 ? -x : x; }

// K directions in lockstep: one value and K derivatives, each derivative
// formed by exactly the operations Dual uses, so direction j of a DualV is
// bit for bit the Dual of direction j -- the value's work is shared.
template <int K>
struct DualV {
    double v, d[K];
    __device__ __forceinline__ DualV() : v(0) {
#pragma unroll
        for (int j = 0; j < K; ++j) d[j] = 0;
    }
    __device__ __forceinline__ DualV(double x) : v(x) {
#pragma unroll
        for (int j = 0; j < K; ++j) d[j] = 0;
    }
};

template <int K> __device__ __forceinline__ DualV<K> operator+(DualV<K> a, DualV<K> b) {
    DualV<K> r(a.v + b.v);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = a.d[j] + b.d[j];
    return r;
}
template <int K> __device__ __forceinline__ DualV<K> operator-(DualV<K> a, DualV<K> b) {
    DualV<K> r(a.v - b.v);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = a.d[j] - b.d[j];
    return r;
}
template <int K> __device__ __forceinline__ DualV<K> operator-(DualV<K> a) {
    DualV<K> r(-a.v);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = -a.d[j];
    return r;
}
template <int K> __device__ __forceinline__ DualV<K> operator*(DualV<K> a, DualV<K> b) {
    DualV<K> r(a.v * b.v);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = a.d[j] * b.v + a.v * b.d[j];
    return r;
}
template <int K> __device__ __forceinline__ DualV<K> operator/(DualV<K> a, DualV<K> b) {
    const double q = a.v / b.v;
    DualV<K> r(q);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = (a.d[j] - q * b.d[j]) / b.v;
    return r;
}
template <int K> __device__ __forceinline__ DualV<K>& operator+=(DualV<K>& a, DualV<K> b) { return a = a + b; }
template <int K> __device__ __forceinline__ DualV<K>& operator-=(DualV<K>& a, DualV<K> b) { return a = a - b; }
template <int K> __device__ __forceinline__ DualV<K>& operator*=(DualV<K>& a, DualV<K> b) { return a = a * b; }
template <int K> __device__ __forceinline__ bool operator<(DualV<K> a, DualV<K> b) { return a.v < b.v; }
template <int K> __device__ __forceinline__ bool operator>(DualV<K> a, DualV<K> b) { return a.v > b.v; }
template <int K> __device__ __forceinline__ bool operator<=(DualV<K> a, DualV<K> b) { return a.v <= b.v; }
template <int K> __device__ __forceinline__ bool operator>=(DualV<K> a, DualV<K> b) { return a.v >= b.v; }
template <int K> __device__ __forceinline__ DualV<K> dsqrt(DualV<K> x) {
    const double s = sqrt(x.v);
    DualV<K> r(s);
#pragma unroll
    for (int j = 0; j < K; ++j) r.d[j] = x.d[j] / (2.0 * s);
    return r;
}
template <int K> __device__ __forceinline__ DualV<K> dabs(DualV<K> x) { return x.v < 0 ? -x : x; }

}  // namespace dev
}  // namespace afx
