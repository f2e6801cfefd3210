// af3d_adjoint.cuh -- pieces shared by the adjoint kernels (af3d_adjoint.cu, compiled like the
// exact step with -fmad=false because its contact re-evaluation must take the forward's
// branches, and af3d_adjoint_rot.cu, the reverse of the predictor, which takes no branch on
// values it recomputes and is compiled with contracted multiply-adds).
#pragma once

#include "af3d_physics.cuh"

namespace af3d {

namespace {

constexpr int kAdjBlock = 128;
inline unsigned blocks(long n) { return (unsigned)((n + kAdjBlock - 1) / kAdjBlock); }

__device__ __forceinline__ V3 ld3(const Planes &P, int x, long s) { return mk(P.p[x][s], P.p[x + 1][s], P.p[x + 2][s]); }
__device__ __forceinline__ void st3(const Planes &P, int x, long s, V3 v) {
  P.p[x][s] = v.x;
  P.p[x + 1][s] = v.y;
  P.p[x + 2][s] = v.z;
}
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(double k, V3 a) { return mk(k * a.x, k * a.y, k * a.z); }
__device__ __forceinline__ V3 &operator+=(V3 &a, V3 b) {
  a.x += b.x; a.y += b.y; a.z += b.z;
  return a;
}
__device__ __forceinline__ V3 &operator-=(V3 &a, V3 b) {
  a.x -= b.x; a.y -= b.y; a.z -= b.z;
  return a;
}
// Products of the reverse pass, with explicit multiply-adds: they form derivatives only (no
// branch depends on them), so they need not repeat the forward's rounding.
__device__ __forceinline__ double dot(V3 a, V3 b) { return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ V3 madd(double k, V3 a, V3 y) {   // y + k a
  return mk(fma(k, a.x, y.x), fma(k, a.y, y.y), fma(k, a.z, y.z));
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return mk(fma(a.y, b.z, -(a.z * b.y)), fma(a.z, b.x, -(a.x * b.z)), fma(a.x, b.y, -(a.y * b.x)));
}
__device__ __forceinline__ void atomic_add3(const Planes &P, int x, long s, V3 v) {
  atomicAdd(&P.p[x][s], v.x);
  atomicAdd(&P.p[x + 1][s], v.y);
  atomicAdd(&P.p[x + 2][s], v.z);
}

// Adjoint planes (one FP64 plane per scalar).
enum AdjPlane : int { AR = 0, AV = 3, AW = 6, ARM = 9, AA = 18, AAL = 21, NADJ = 24 };   // state adjoint
enum AccPlane : int { CR = 0, CV = 3, CW = 6, CS = 9, NACC = 21 };                          // scattered parts

// Sphere patterns of init_Verlet.cu:130-142.
__device__ __forceinline__ V3 pattern(int k) {
  switch (k) {
    case 0: return mk(1.0, 1.0, 1.0);
    case 1: return mk(1.0, -1.0, -1.0);
    case 2: return mk(-1.0, -1.0, 1.0);
    default: return mk(-1.0, 1.0, -1.0);
  }
}

// Folds the sphere-centre adjoints s_b[k] (s_k = r1 + pos R1 p_k) into r1_b and the rows of R1_b.
__device__ __forceinline__ void fold_spheres(const Planes &acc, long s, double pos, V3 &r1_b, V3 *Rb) {
  for (int k = 0; k < 4; k++) {
    const V3 sb = ld3(acc, CS + 3 * k, s), p = pattern(k);
    r1_b += sb;
    Rb[0] += (pos * sb.x) * p;
    Rb[1] += (pos * sb.y) * p;
    Rb[2] += (pos * sb.z) * p;
  }
}

}  // namespace

}  // namespace af3d
