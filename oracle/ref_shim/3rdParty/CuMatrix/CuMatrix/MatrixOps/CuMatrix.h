// Checker-build stand-in for CuMatrix's MatrixOps/CuMatrix.h — TEST INFRASTRUCTURE ONLY.
//
// The reference's VBD kernels call small vector / matrix helpers of its CuMatrix
// submodule, which is empty in the reference tree (no pinned commit). Each helper below
// is written from its name and its uses in VBD/VBDPhysicsCompute.cu and
// VBD/VBD_GeneralCompute.h, with these conventions:
//   * vec3X(a, b, out) / vec9X: element-wise, out may alias an input;
//   * vecNMulAddTo(a, s, out): out += s * a;   vec3Mul(a, s, out): out = s * a;
//   * matrices are column-major arrays (element (r, c) of an R x C matrix at c * R + r):
//     the uses fix it (T_3x2 in accumulateBoundaryForceAndHessianGPU sets column 0 at
//     indices 0..2, column 1 at 3..5; F = Ds * DmInv with Ds built from three column
//     vectors; DmInv read column by column);
//   * faceNormal(A, B, C, n): the unit normal (B - A) x (C - A) / |...|;
//   * Mat9x9Static<T>: 81 values with operator()(row, col) and multiplyBy(s).
// The 3x3 PSD solve (solve3x3_psd_stable) is not used by the functions this build checks.
#pragma once
#include <cmath>
#include <cstdint>

#ifndef GPU_CPU_INLINE_FUNC
#define GPU_CPU_INLINE_FUNC inline
#endif
#ifndef SQR
#define SQR(x) ((x) * (x))
#endif

namespace CuMatrix {

template <typename T>
inline void vec3Set(T* out, const T* in) { out[0] = in[0]; out[1] = in[1]; out[2] = in[2]; }
template <typename T, typename X, typename Y, typename Z>
inline void vec3Set(T* out, X x, Y y, Z z) { out[0] = T(x); out[1] = T(y); out[2] = T(z); }
template <typename T>
inline void vec3Minus(const T* a, const T* b, T* out) { out[0] = a[0] - b[0]; out[1] = a[1] - b[1]; out[2] = a[2] - b[2]; }
template <typename T>
inline void vec3Add(const T* a, const T* b, T* out) { out[0] = a[0] + b[0]; out[1] = a[1] + b[1]; out[2] = a[2] + b[2]; }
template <typename T, typename S>
inline void vec3Mul(const T* a, S s, T* out) { out[0] = a[0] * s; out[1] = a[1] * s; out[2] = a[2] * s; }
template <typename T, typename S>
inline void vec3MulAddTo(const T* a, S s, T* out) { out[0] += a[0] * s; out[1] += a[1] * s; out[2] += a[2] * s; }
template <typename T>
inline T vec3DotProduct(const T* a, const T* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename T>
inline T vec3NormSquare(const T* a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }
template <typename T>
inline T vec3Norm(const T* a) { return std::sqrt(vec3NormSquare(a)); }
template <typename T>
inline void vec3Normalize(T* a) { const T n = vec3Norm(a); a[0] /= n; a[1] /= n; a[2] /= n; }
template <typename T>
inline void vec3CrossProduct(const T* a, const T* b, T* out) {
    const T x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    out[0] = x; out[1] = y; out[2] = z;
}
template <typename T, typename S>
inline void vec3lerp(const T* a, S t, const T* d, T* out) { out[0] = a[0] + t * d[0]; out[1] = a[1] + t * d[1]; out[2] = a[2] + t * d[2]; }
template <typename T>
inline void vec3OuterProduct(const T* a, const T* b, T* out) {
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) out[3 * c + r] = a[r] * b[c];
}
template <typename T>
inline T vec2Norm(const T* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1]); }
template <typename T, typename S>
inline void vec9Mul(const T* a, S s, T* out) { for (int i = 0; i < 9; ++i) out[i] = a[i] * s; }
template <typename T>
inline void vec9Add(const T* a, const T* b, T* out) { for (int i = 0; i < 9; ++i) out[i] = a[i] + b[i]; }
template <typename T, typename S>
inline void vec9MulAddTo(const T* a, S s, T* out) { for (int i = 0; i < 9; ++i) out[i] += a[i] * s; }

template <typename T>
inline void mat3MatProduct(const T* A, const T* B, T* C) {
    T out[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) out[3 * c + r] = A[r] * B[3 * c] + A[3 + r] * B[3 * c + 1] + A[6 + r] * B[3 * c + 2];
    for (int i = 0; i < 9; ++i) C[i] = out[i];
}
template <typename T>
inline void mat3VecProduct(const T* M, const T* v, T* out) {
    T o[3];
    for (int r = 0; r < 3; ++r) o[r] = M[r] * v[0] + M[3 + r] * v[1] + M[6 + r] * v[2];
    out[0] = o[0]; out[1] = o[1]; out[2] = o[2];
}
template <typename T>
inline T mat3Determinant(const T* F) {
    return F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) + F[6] * (F[1] * F[5] - F[4] * F[2]);
}
template <typename T>
inline T mat3FNormSquare(const T* F) {
    T s = 0;
    for (int i = 0; i < 9; ++i) s += F[i] * F[i];
    return s;
}

template <typename T, int R, int C>
inline T& accessMatElement(T* m, int r, int c) { return m[c * R + r]; }
template <typename T, int R, int C>
inline const T& accessMatElement(const T* m, int r, int c) { return m[c * R + r]; }

// C (M x K) = A (M x N) * B (N x K), all column-major.
template <typename T, int M, int N, int K>
inline void matMulMxN(const T* A, const T* B, T* Cout) {
    for (int k = 0; k < K; ++k)
        for (int m = 0; m < M; ++m) {
            T s = 0;
            for (int n = 0; n < N; ++n) s += A[n * M + m] * B[k * N + n];
            Cout[k * M + m] = s;
        }
}

template <typename T>
struct Mat9x9Static {
    T data[81];
    T& operator()(int r, int c) { return data[c * 9 + r]; }
    const T& operator()(int r, int c) const { return data[c * 9 + r]; }
    template <typename S>
    void multiplyBy(S s) { for (int i = 0; i < 81; ++i) data[i] *= s; }
};
template <typename T>
using Mat9x9Abstract = Mat9x9Static<T>;

template <typename T>
inline void vec9OuterProduct(const T* a, const T* b, Mat9x9Static<T>& M) {
    for (int c = 0; c < 9; ++c)
        for (int r = 0; r < 9; ++r) M(r, c) = a[r] * b[c];
}

template <typename T>
inline void faceNormal(const T* A, const T* B, const T* C, T* n) {
    T e1[3], e2[3];
    vec3Minus(B, A, e1);
    vec3Minus(C, A, e2);
    vec3CrossProduct(e1, e2, n);
    vec3Normalize(n);
}

}  // namespace CuMatrix
