// af3d_kernels.cu -- the step kernels (compiled with -fmad=false: see af3d_physics.cuh).
//
// Kernels, per step of the fused path (af3d_step):
//   k_predict      init_Verlet (+ cell key, bucket count)              one thread per clump
//   (cells)        scan of bucket counts, scatter, deterministic rank  af3d_cells.cu
//   k_permute      move every plane into (cell, id) order, build the packed neighbour records
//   k_lists_forces each block builds its clumps' contact item lists (neighbour walk, FP32
//                  culling, exact overlap tests, boundary gates), then runs boundaries + sphere
//                  contacts + bed + get_accel + finish_Verlet for them, gathering (never
//                  scattering) contributions: no atomics on forces
// The per-routine C-ABI entry points use k_boundary / k_part / k_get_accel / k_finish_verlet,
// which apply the same device functions to the F, T planes one routine at a time.
#include <algorithm>
#include <cfloat>

#include "af3d_cellwalk.cuh"

namespace af3d {

namespace {

constexpr int kBlock = 128;   // the per-clump kernels other than the fused force kernel

inline unsigned grid_for(long n, int block = kBlock) {
  return (unsigned)((n + block - 1) / block);
}

__device__ __forceinline__ V3 load3(const Planes &P, int x, long s) {
  return mk(P.p[x][s], P.p[x + 1][s], P.p[x + 2][s]);
}
__device__ __forceinline__ void store3(const Planes &P, int x, long s, V3 v) {
  P.p[x][s] = v.x;
  P.p[x + 1][s] = v.y;
  P.p[x + 2][s] = v.z;
}

__device__ __forceinline__ void raise_status(DevScalars *d, int err) {
  atomicOr(&d->status, 1 << err);
}

// ------------------------------------------------------------------ import / export

// keep_order: slot s keeps the clump it holds (id[s]); otherwise slot s receives clump s.
__global__ void k_aos_to_planes(const af3d_particle *__restrict__ aos, const double *__restrict__ acc,
                                const double *__restrict__ anga, const int *__restrict__ flume_of_id,
                                Planes P, long long *id, int *flume, bool keep_order, long s0, long n) {
  long s = s0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const long long i = keep_order ? id[s] : s;
  const af3d_particle &q = aos[i];
  store3(P, RX, s, mk(q.rr.x, q.rr.y, q.rr.z));
  store3(P, VX, s, mk(q.vv.x, q.vv.y, q.vv.z));
  store3(P, WX, s, mk(q.ww.x, q.ww.y, q.ww.z));
  store3(P, R00, s, mk(q.Rmatx.x, q.Rmatx.y, q.Rmatx.z));
  store3(P, R10, s, mk(q.Rmaty.x, q.Rmaty.y, q.Rmaty.z));
  store3(P, R20, s, mk(q.Rmatz.x, q.Rmatz.y, q.Rmatz.z));
  for (int k = 0; k < 4; k++) store3(P, S0X + 3 * k, s, mk(q.rr_s[k].x, q.rr_s[k].y, q.rr_s[k].z));
  V3 a = acc ? mk(acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]) : mk(0.0, 0.0, 0.0);
  V3 al = anga ? mk(anga[3 * i], anga[3 * i + 1], anga[3 * i + 2]) : mk(0.0, 0.0, 0.0);
  store3(P, AIX, s, a);
  store3(P, ALIX, s, al);
  store3(P, AFX, s, mk(0.0, 0.0, 0.0));
  store3(P, ALFX, s, mk(0.0, 0.0, 0.0));
  store3(P, FX, s, mk(0.0, 0.0, 0.0));
  store3(P, TX, s, mk(0.0, 0.0, 0.0));
  const double r = q.radius, rho = q.density;
  P.p[RAD][s] = r;
  P.p[DEN][s] = rho;
  P.p[MASS][s] = q.mass;
  store3(P, IXX, s, mk(q.moment_of_inertia.x, q.moment_of_inertia.y, q.moment_of_inertia.z));
  P.p[MSPH][s] = kSPH_FACT * rho * r * r * r;   // force_part.cu:58
  P.p[MWALL][s] = kSPH_FACT * r * r * r * rho;  // force_walls.cu:47
  P.p[ADRAG][s] = drag_factor(r, q.mass);       // get_accel.cu:47
  P.p[IMASS][s] = 1.0 / q.mass;
  P.p[IINER][s] = 1.0 / q.moment_of_inertia.x;
  id[s] = i;
  flume[s] = flume_of_id[i];
}

__global__ void k_planes_to_aos(Planes P, const long long *__restrict__ id, const int *__restrict__ flume,
                                af3d_particle *aos, double *acc, double *anga, const DevScalars *d,
                                long s0, long n) {
  long s = s0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const af3d_system_par &sy = d->flumes[flume[s]].sys;
  const double cost = sy.cost, sint = sy.sint;
  af3d_particle &q = aos[id[s]];
  q.radius = P.p[RAD][s];
  q.mass = P.p[MASS][s];
  q.density = P.p[DEN][s];
  V3 I = load3(P, IXX, s);
  q.moment_of_inertia = {I.x, I.y, I.z};
  V3 r = load3(P, RX, s);
  q.rr = {r.x, r.y, r.z};
  V3 rr = to_slope(r, cost, sint);
  q.rrot = {rr.x, rr.y, rr.z};
  for (int k = 0; k < 4; k++) {
    V3 sk = load3(P, S0X + 3 * k, s);
    q.rr_s[k] = {sk.x, sk.y, sk.z};
    V3 qk = to_slope(sk, cost, sint);
    q.rrot_s[k] = {qk.x, qk.y, qk.z};
  }
  V3 v = load3(P, VX, s), w = load3(P, WX, s);
  q.vv = {v.x, v.y, v.z};
  q.ww = {w.x, w.y, w.z};
  V3 a = load3(P, R00, s), b = load3(P, R10, s), c = load3(P, R20, s);
  q.Rmatx = {a.x, a.y, a.z};
  q.Rmaty = {b.x, b.y, b.z};
  q.Rmatz = {c.x, c.y, c.z};
  if (acc) {
    V3 ai = load3(P, AIX, s);
    acc[3 * id[s]] = ai.x; acc[3 * id[s] + 1] = ai.y; acc[3 * id[s] + 2] = ai.z;
  }
  if (anga) {
    V3 al = load3(P, ALIX, s);
    anga[3 * id[s]] = al.x; anga[3 * id[s] + 1] = al.y; anga[3 * id[s] + 2] = al.z;
  }
}

// ------------------------------------------------------------------ neighbour records

__device__ __forceinline__ float f_up(double x) { return to_float_ru(x); }

// Packed FP64 neighbour record and conservative FP32 culling record of one clump.
// The culling bounds are formed in FP32 from the FP32-rounded coordinates.  M32 = max |coordinate|
// in FP32 is within 2^-24 of the FP64 maximum M, so mu = 2^-22 * M32 * (1 + 2^-20) is at least
// 4 x 2^-24 M: the FP32 difference of a coordinate of this clump and one of a partner is within
// 2^-24 (M + M') (the two roundings) + 2^-24 |difference| of the exact one, so a distance formed
// from FP32 coordinates errs by at most sqrt(3) 2^-24 (M + M') + 2^-24 d < mu + mu' + 2^-24 d,
// and the last term is covered by the tests' relative slack (1 + 2^-18) on squared bounds.  The
// sphere extent ext32 = max_k |s_k - r| from the FP32 coordinates is within 2 sqrt(3) 2^-24 M + a
// few 2^-24 ext of the exact one, which the added 2 mu and the factor (1 + 2^-20) cover.
__device__ __forceinline__ void make_records(V3 r, V3 v, V3 w, const V3 *sp, double rad, double msph,
                                             double mwall, NbrRec &q, CullRec &c) {
  q.rx = r.x; q.ry = r.y; q.rz = r.z;
  q.vx = v.x; q.vy = v.y; q.vz = v.z;
  q.wx = w.x; q.wy = w.y; q.wz = w.z;
  for (int k = 0; k < 4; k++) {
    q.s[3 * k] = sp[k].x; q.s[3 * k + 1] = sp[k].y; q.s[3 * k + 2] = sp[k].z;
  }
  q.rad = rad; q.msph = msph; q.mwall = mwall;
  const float cx = to_float_rn(r.x), cy = to_float_rn(r.y), cz = to_float_rn(r.z);
  float M = fmaxf(fmaxf(fabsf(cx), fabsf(cy)), fabsf(cz));
  float ext = 0.0f;
  float4 sf[4];
  for (int k = 0; k < 4; k++) {
    sf[k] = make_float4(to_float_rn(sp[k].x), to_float_rn(sp[k].y), to_float_rn(sp[k].z), 0.0f);
    M = fmaxf(M, fmaxf(fmaxf(fabsf(sf[k].x), fabsf(sf[k].y)), fabsf(sf[k].z)));
    const float dx = sf[k].x - cx, dy = sf[k].y - cy, dz = sf[k].z - cz;
    ext = fmaxf(ext, sqrtf(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx))));
  }
  const float radf = f_up(rad);
  // 2^-22 * max|coordinate|: see above.
  const float mu = fmaxf(M, radf) * 2.384185791015625e-07f * (1.0f + 9.5367431640625e-07f) + 1e-30f;
  const float sph = radf * (1.0f + 9.5367431640625e-07f) + mu;
  c.c = make_float4(cx, cy, cz, (ext * (1.0f + 9.5367431640625e-07f) + 2.0f * mu) + sph);
  for (int k = 0; k < 4; k++) c.s[k] = make_float4(sf[k].x, sf[k].y, sf[k].z, sph);
}

constexpr int kPermBlock = 128;
// Records are staged in shared memory with an odd stride (25 doubles) so that the per-thread
// writes of a 24-double record hit distinct banks.
constexpr int kRecWords = (int)(sizeof(NbrRec) / 8);   // 24
constexpr int kRecStride = kRecWords + 1;

// One thread's neighbour record into the block's shared-memory staging.
__device__ __forceinline__ void stage_nbr_record(const NbrRec &q, double *s_nbr) {
  const double *qw = reinterpret_cast<const double *>(&q);
#pragma unroll
  for (int k = 0; k < kRecWords; k++) s_nbr[threadIdx.x * kRecStride + k] = qw[k];
}

// One thread's records into the block's shared-memory staging.
__device__ __forceinline__ void stage_record(const NbrRec &q, const CullRec &cr, double *s_nbr, CullRec *s_cull) {
  stage_nbr_record(q, s_nbr);
  s_cull[threadIdx.x] = cr;
}

// The block's staged neighbour records written out as contiguous 16-byte stores (after a
// barrier that follows the staging).
template <int NB>
__device__ __forceinline__ void copy_nbr_records(long base, long n, NbrRec *nbr, const double *s_nbr) {
  const long cnt = n - base < NB ? n - base : NB;
  const int nw = (int)(cnt * kRecWords) / 2;   // double2 words of the block's records
  double2 *b = reinterpret_cast<double2 *>(nbr + base);
  for (int i = threadIdx.x; i < nw; i += NB) {
    const int w0 = 2 * i, r0 = w0 / kRecWords, k0 = w0 - r0 * kRecWords;   // k0 even, k0 + 1 < 24
    b[i] = make_double2(s_nbr[r0 * kRecStride + k0], s_nbr[r0 * kRecStride + k0 + 1]);
  }
}

// ... and the culling records with them.
template <int NB>
__device__ __forceinline__ void copy_records(long base, long n, NbrRec *nbr, CullRec *cull, const double *s_nbr,
                                             const CullRec *s_cull) {
  copy_nbr_records<NB>(base, n, nbr, s_nbr);
  const long cnt = n - base < NB ? n - base : NB;
  const int m16 = (int)(cnt * (long)(sizeof(CullRec) / 16));
  const float4 *c = reinterpret_cast<const float4 *>(s_cull);
  float4 *e = reinterpret_cast<float4 *>(cull + base);
  for (int i = threadIdx.x; i < m16; i += NB) e[i] = c[i];
}

// The block's records, staged in shared memory and written out as contiguous 16-byte stores.
// Every thread of an NB-thread block calls this (slots past n contribute nothing).
template <int NB>
__device__ __forceinline__ void store_records(bool valid, long base, long n, const NbrRec &q, const CullRec &cr,
                                              NbrRec *nbr, CullRec *cull, double *s_nbr, CullRec *s_cull) {
  if (valid) stage_record(q, cr, s_nbr, s_cull);
  __syncthreads();
  copy_records<NB>(base, n, nbr, cull, s_nbr, s_cull);
}

// ------------------------------------------------------------------ init_Verlet (+ cell keys)

// Cell coordinate of cells.cu:69-77 (multiplication by cs_inv, then `== ncell -> ncell-1`).
__device__ __forceinline__ long bin_axis(double x, double xmin, double inv, long n) {
  long i = (long)trunc_to_ll(inv * (x - xmin));
  if (i == n) i--;
  return i;
}

constexpr double kSmallAngle2 = 9.765625e-04;   // (2^-5)^2

// init_Verlet.cu:25-148 for one clump that is not removed: r, v, w and the rotation rows move
// one step with a_i, alpha_i; sp receives the new sphere centres.
__device__ __forceinline__ void predict_state(V3 &r, V3 &v, V3 &w, V3 a, V3 al, V3 &Rx, V3 &Ry, V3 &Rz, V3 *sp,
                                              double rad, double dt, double hdt) {
  r.x += dt * (v.x + hdt * a.x);
  r.y += dt * (v.y + hdt * a.y);
  r.z += dt * (v.z + hdt * a.z);
  v.x += dt * a.x;
  v.y += dt * a.y;
  v.z += dt * a.z;
  V3 dO = mk(dt * (w.x + hdt * al.x), dt * (w.y + hdt * al.y), dt * (w.z + hdt * al.z));
  const double mag2 = dO.x * dO.x + dO.y * dO.y + dO.z * dO.z;
  double mag, imag = 0.0;
  V3 dRx, dRy, dRz;
  if (kFast && in_open_range_bits(mag2, 0.0, kSmallAngle2)) {
    // Fast mode, |dO| < 2^-5: the Rodrigues matrix c I + (sin/|dO|) [dO]x + ((1-c)/|dO|^2) dO dO^T
    // from the Maclaurin series of sin(t)/t and (1 - cos t)/t^2 in t^2 = |dO|^2 (truncated
    // after t^8 and t^10: the first omitted terms are below 2^-53 of the sums), no square
    // root, sine or cosine.
    // Horner form in t2 with the series' coefficients (1/6, 1/120, 1/5040, 1/362880 and
    // 1/2, 1/24, 1/720, 1/40320, 1/3628800): four multiply-adds each.
    // Below |dO| = 2^-10 (t2 < 2^-20, the usual case) the series end after t^4: the first
    // omitted terms, t^6 / 5040 and t^6 / 40320, are below 2^-72.
    const double t2 = mag2;
    double A, Bq;
    if (in_open_range_bits(t2, 0.0, 9.5367431640625e-07)) {
      A = 1.0 + t2 * (-1.0 / 6.0 + t2 * (1.0 / 120.0));
      Bq = 0.5 + t2 * (-1.0 / 24.0 + t2 * (1.0 / 720.0));
    } else {
      A = 1.0 + t2 * (-1.0 / 6.0 + t2 * (1.0 / 120.0 + t2 * (-1.0 / 5040.0 + t2 * (1.0 / 362880.0))));
      Bq = 0.5 + t2 * (-1.0 / 24.0 + t2 * (1.0 / 720.0 + t2 * (-1.0 / 40320.0 + t2 * (1.0 / 3628800.0))));
    }
    const double cc = 1.0 - t2 * Bq;
    const V3 sv = mk(A * dO.x, A * dO.y, A * dO.z);
    const V3 bv = mk(Bq * dO.x, Bq * dO.y, Bq * dO.z);
    dRx = mk(bv.x * dO.x + cc, bv.x * dO.y - sv.z, bv.x * dO.z + sv.y);
    dRy = mk(bv.y * dO.x + sv.z, bv.y * dO.y + cc, bv.y * dO.z - sv.x);
    dRz = mk(bv.z * dO.x - sv.y, bv.z * dO.y + sv.x, bv.z * dO.z + cc);
  } else {
    if (kFast) {
      imag = rsqrt(mag2);
      mag = mag2 * imag;
    } else {
      mag = sqrt(mag2);
    }
    if (mag > 0.0) {
      // Rodrigues rotation about dO/|dO| by |dO| (init_Verlet.cu:63-83)
      V3 u;
      double c, sn;
      if (kFast) {
        u = mk(dO.x * imag, dO.y * imag, dO.z * imag);
        sincos(mag, &sn, &c);
      } else {
        u = mk(dO.x / mag, dO.y / mag, dO.z / mag);
        sincos(mag, &sn, &c);   // init_Verlet.cu's cos and sin, from one argument reduction
      }
      const double omc = 1.0 - c;
      dRx = mk(omc * u.x * u.x + c, omc * u.x * u.y - sn * u.z, omc * u.x * u.z + sn * u.y);
      dRy = mk(omc * u.y * u.x + sn * u.z, omc * u.y * u.y + c, omc * u.y * u.z - sn * u.x);
      dRz = mk(omc * u.z * u.x - sn * u.y, omc * u.z * u.y + sn * u.x, omc * u.z * u.z + c);
    } else {
      dRx = mk(1.0, 0.0, 0.0);
      dRy = mk(0.0, 1.0, 0.0);
      dRz = mk(0.0, 0.0, 1.0);
    }
  }
  // R <- dR R (rows), then each column renormalised (init_Verlet.cu:92-114)
  V3 Tx = mk(dRx.x * Rx.x + dRx.y * Ry.x + dRx.z * Rz.x, dRx.x * Rx.y + dRx.y * Ry.y + dRx.z * Rz.y,
             dRx.x * Rx.z + dRx.y * Ry.z + dRx.z * Rz.z);
  V3 Ty = mk(dRy.x * Rx.x + dRy.y * Ry.x + dRy.z * Rz.x, dRy.x * Rx.y + dRy.y * Ry.y + dRy.z * Rz.y,
             dRy.x * Rx.z + dRy.y * Ry.z + dRy.z * Rz.z);
  V3 Tz = mk(dRz.x * Rx.x + dRz.y * Ry.x + dRz.z * Rz.x, dRz.x * Rx.y + dRz.y * Ry.y + dRz.z * Rz.y,
             dRz.x * Rx.z + dRz.y * Ry.z + dRz.z * Rz.z);
  if (kFast) {
    // 1/sqrt(n2) for a column norm n2 within 2^-26 of 1 (a rotation times a rotation):
    // one Newton step from 1, 1.5 - n2/2, whose error 3/8 (n2 - 1)^2 is below 2^-54.
    auto inv_norm = [](double n2) {   // |n2 - 1| < 2^-26, tested on the bits
      return in_open_range_bits(n2, 1.0 - 1.4901161193847656e-08, 1.0 + 1.4901161193847656e-08) ? 1.5 - 0.5 * n2
                                                                                                 : rsqrt(n2);
    };
    double in = inv_norm(Tx.x * Tx.x + Ty.x * Ty.x + Tz.x * Tz.x);
    Rx.x = Tx.x * in; Ry.x = Ty.x * in; Rz.x = Tz.x * in;
    in = inv_norm(Tx.y * Tx.y + Ty.y * Ty.y + Tz.y * Tz.y);
    Rx.y = Tx.y * in; Ry.y = Ty.y * in; Rz.y = Tz.y * in;
    in = inv_norm(Tx.z * Tx.z + Ty.z * Ty.z + Tz.z * Tz.z);
    Rx.z = Tx.z * in; Ry.z = Ty.z * in; Rz.z = Tz.z * in;
  } else {
    double nrm = sqrt(Tx.x * Tx.x + Ty.x * Ty.x + Tz.x * Tz.x);
    Rx.x = Tx.x / nrm; Ry.x = Ty.x / nrm; Rz.x = Tz.x / nrm;
    nrm = sqrt(Tx.y * Tx.y + Ty.y * Ty.y + Tz.y * Tz.y);
    Rx.y = Tx.y / nrm; Ry.y = Ty.y / nrm; Rz.y = Tz.y / nrm;
    nrm = sqrt(Tx.z * Tx.z + Ty.z * Ty.z + Tz.z * Tz.z);
    Rx.z = Tx.z / nrm; Ry.z = Ty.z / nrm; Rz.z = Tz.z / nrm;
  }
  w.x += dt * al.x;
  w.y += dt * al.y;
  w.z += dt * al.z;
  // sphere centres r + (radius/sqrt2) R (+-1,+-1,+-1) (init_Verlet.cu:130-142)
  const double pos = kFast ? rad * (1.0 / kROOT2) : rad / kROOT2;
  if (kFast) {
    // the four patterns (a + c, b - c, c - a, -(b + c)) with a = x + y, b = x - y, from the
    // two partial sums r0 + pos c and r0 - pos c: eight operations per row
    auto row = [&](double r0, const V3 &R, double &s0, double &s1, double &s2, double &s3) {
      const double a = R.x + R.y, b = R.x - R.y;
      const double up = r0 + pos * R.z, dn = r0 - pos * R.z;
      s0 = up + pos * a;
      s2 = up - pos * a;
      s1 = dn + pos * b;
      s3 = dn - pos * b;
    };
    row(r.x, Rx, sp[0].x, sp[1].x, sp[2].x, sp[3].x);
    row(r.y, Ry, sp[0].y, sp[1].y, sp[2].y, sp[3].y);
    row(r.z, Rz, sp[0].z, sp[1].z, sp[2].z, sp[3].z);
    return;
  }
  sp[0] = mk(r.x + pos * (Rx.x + Rx.y + Rx.z), r.y + pos * (Ry.x + Ry.y + Ry.z), r.z + pos * (Rz.x + Rz.y + Rz.z));
  sp[1] = mk(r.x + pos * (Rx.x - Rx.y - Rx.z), r.y + pos * (Ry.x - Ry.y - Ry.z), r.z + pos * (Rz.x - Rz.y - Rz.z));
  sp[2] = mk(r.x + pos * (-Rx.x - Rx.y + Rx.z), r.y + pos * (-Ry.x - Ry.y + Ry.z),
             r.z + pos * (-Rz.x - Rz.y + Rz.z));
  sp[3] = mk(r.x + pos * (-Rx.x + Rx.y - Rx.z), r.y + pos * (-Ry.x + Ry.y - Ry.z),
             r.z + pos * (-Rz.x + Rz.y - Rz.z));
}

// cell_locate's bucket of a clump at r (cells.cu:60-92) at time t: the flume's cell offset + cell
// index, or ncell_total + id for a clump that is not binned (removed, or non-finite).
__device__ __forceinline__ long bucket_key(V3 r, const DevFlume &fl, DevScalars *d, long long id, double t) {
  const af3d_cell_par &g = fl.grid;
  if (is_removed(t, r.x, fl.sys.side.x)) return d->ncell_total + id;
  if (!(finite_bits(r.x) && finite_bits(r.y) && finite_bits(r.z))) {
    raise_status(d, AF3D_ERR_NAN);
    return d->ncell_total + id;
  }
  long i = bin_axis(r.x, g.rr_min.x, g.cs_inv.x, g.ncell.x);
  long j = bin_axis(r.y, g.rr_min.y, g.cs_inv.y, g.ncell.y);
  long k = bin_axis(r.z, g.rr_min.z, g.cs_inv.z, g.ncell.z);
  if (i < 0 || j < 0 || k < 0) {
    raise_status(d, AF3D_ERR_NEGATIVE_CELL);
    i = i < 0 ? 0 : i; j = j < 0 ? 0 : j; k = k < 0 ? 0 : k;
  }
  if (i >= g.ncell.x || j >= g.ncell.y || k >= g.ncell.z) {
    raise_status(d, AF3D_ERR_GRID_ESCAPE);
    i = i < g.ncell.x ? i : g.ncell.x - 1;
    j = j < g.ncell.y ? j : g.ncell.y - 1;
    k = k < g.ncell.z ? k : g.ncell.z - 1;
  }
  return fl.cell_off + i + g.ncell.x * (j + k * g.ncell.y);
}

// init_Verlet.cu:25-148 for one clump (PREDICT), and/or cell_locate's binning (cells.cu:60-92)
// with the current time (KEYS): the bucket key, the bucket count and the clump's arrival rank.
// Clumps that are not binned (removed, or non-finite) get the unique bucket ncell_total + id, so every
// bucket holds its clumps in id order after the rank pass.  `t_prev`: init_Verlet's removal test
// uses the time before the advance (the fused step advances time first).  RECORDS: also write
// the clump's neighbour records at its own slot (steps that keep the slot order).
template <bool PREDICT, bool KEYS, bool RECORDS>
__global__ void __launch_bounds__(kBlock) k_predict(Planes P, DevScalars *d, bool t_prev, Cells cells,
                                                    const long long *__restrict__ id,
                                                    const int *__restrict__ flume, NbrRec *nbr,
                                                    CullRec *cull, long s0, long n) {
  __shared__ double s_nbr[RECORDS ? kPermBlock * kRecStride : 1];
  __shared__ CullRec s_cull[RECORDS ? kPermBlock : 1];
  const long base = s0 + blockIdx.x * (long)blockDim.x;
  const long s = base + threadIdx.x;
  const bool valid = s < n;
  if (!RECORDS && !valid) return;
  NbrRec q;
  CullRec cr;
  if (valid) {
    const DevFlume &fl = d->flumes[flume[s]];
    V3 r = load3(P, RX, s);
    V3 v, w, sp[4];
    bool have = false;   // v, w, sp hold the clump's current values
    if (PREDICT) {
      const double t_init = t_prev ? d->time_prev : d->time;
      if (is_removed(t_init, r.x, fl.sys.side.x)) {
        P.p[RAD][s] = 0.0;
      } else {
        v = load3(P, VX, s);
        w = load3(P, WX, s);
        V3 Rx = load3(P, R00, s), Ry = load3(P, R10, s), Rz = load3(P, R20, s);
        predict_state(r, v, w, load3(P, AIX, s), load3(P, ALIX, s), Rx, Ry, Rz, sp, P.p[RAD][s], fl.sys.dt,
                      fl.sys.hdt);
        store3(P, RX, s, r);
        store3(P, VX, s, v);
        store3(P, WX, s, w);
        store3(P, R00, s, Rx);
        store3(P, R10, s, Ry);
        store3(P, R20, s, Rz);
        for (int k = 0; k < 4; k++) store3(P, S0X + 3 * k, s, sp[k]);
        have = true;
      }
    }
    if (RECORDS) {
      if (!have) {
        v = load3(P, VX, s);
        w = load3(P, WX, s);
        for (int k = 0; k < 4; k++) sp[k] = load3(P, S0X + 3 * k, s);
      }
      make_records(r, v, w, sp, P.p[RAD][s], P.p[MSPH][s], P.p[MWALL][s], q, cr);
    }
    if (KEYS) {
      const long key = bucket_key(r, fl, d, id[s], d->time);
      cells.key[s] = (int)key;
      cells.rank_tmp[s] = arrive_in_bucket(cells, key);
    }
  }
  if (RECORDS) store_records<kPermBlock>(valid, base, n, q, cr, nbr, cull, s_nbr, s_cull);
}

// ------------------------------------------------------------------ permutation + records

// dst[p][s] = src[p][perm[s]] for every plane (the force/torque accumulators and a_f only with
// `ft`: the fused step rewrites them before reading), plus the packed records of the new slot,
// assembled in shared memory and written out as contiguous 16-byte stores.
__global__ void __launch_bounds__(kPermBlock) k_permute(Planes src, Planes dst, const int *__restrict__ perm,
                                                        const long long *__restrict__ id_src,
                                                        long long *id_dst, const int *__restrict__ fl_src,
                                                        int *fl_dst, NbrRec *nbr, CullRec *cull,
                                                        bool ft, long n) {
  __shared__ double s_nbr[kPermBlock * kRecStride];
  __shared__ CullRec s_cull[kPermBlock];
  const long base = blockIdx.x * (long)kPermBlock;
  const long s = base + threadIdx.x;
  if (s < n) {
    if (perm) {
      const long o = perm[s];
#pragma unroll 8
      for (int p = 0; p < NPLANES; p++)
        if (ft || ((p < FX || p > TZ) && (p < AFX || p > ALFZ))) dst.p[p][s] = src.p[p][o];
      id_dst[s] = id_src[o];
      fl_dst[s] = fl_src[o];
    }
  }
  if (!nbr) return;
  NbrRec q;
  CullRec cr;
  if (s < n) {
    V3 sp[4];
    for (int k = 0; k < 4; k++) sp[k] = load3(dst, S0X + 3 * k, s);
    make_records(load3(dst, RX, s), load3(dst, VX, s), load3(dst, WX, s), sp, dst.p[RAD][s], dst.p[MSPH][s],
                 dst.p[MWALL][s], q, cr);
  }
  store_records<kPermBlock>(s < n, base, n, q, cr, nbr, cull, s_nbr, s_cull);
}

// ------------------------------------------------------------------ particle contacts

constexpr int kCandCap = 48;
// The sixteen sph_id passes of force_part for one clump are summed in the reference order:
// sph_id outer, then cells, then slots.  Phase 1 walks the 27 neighbour cells once and keeps the
// FP32-surviving partners with their 16-bit pair masks; phase 2 flattens them into one item list
// per clump in that order (sph_id-major); the items are then run through the exact FP64 test and
// contact law one by one and added in list order.  Returns false when a list would overflow.
constexpr int kItemCap = 96;

__device__ __forceinline__ bool gather_items(long s, const Own &o, const af3d_cell_par &g,
                                             long long off, const CullRec *__restrict__ cull,
                                             const int *__restrict__ start, const int *__restrict__ order,
                                             unsigned want, unsigned *items, int cap, int &nitems) {
  const CullRec me = cull[s];
  const Search q = search_centre(o.r, g, off);
  int cand_t[kCandCap];
  unsigned short cand_m[kCandCap];
  int ncand = 0;
  bool overflow = false;
  for_neighbour_slots_pre(q, g, start, order, [&](int t) {
    if (t == s) return;
    const unsigned m = pair_mask(me, cull[t]) & want;
    if (!m) return;
    if (ncand < kCandCap) {
      cand_t[ncand] = t;
      cand_m[ncand] = (unsigned short)m;
      ncand++;
    } else {
      overflow = true;
    }
  });
  nitems = 0;
  if (overflow) return false;
#pragma unroll 1
  for (int p = 0; p < 16; p++) {
    if (!((want >> p) & 1u)) continue;
#pragma unroll 1
    for (int k = 0; k < ncand; k++) {
      if (!((cand_m[k] >> p) & 1u)) continue;
      if (nitems == cap) return false;
      items[nitems++] = ((unsigned)cand_t[k] << 4) | (unsigned)p;   // (partner slot, sph_id - 1)
    }
  }
  return true;
}

// Every pair of clump s walked cell by cell once per sph_id (the order of sixteen force_part
// launches); used when a clump has more partners than the item lists hold.
__device__ __forceinline__ int contacts_by_pass(long s, const Own &o, const Consts &c,
                                                const af3d_cell_par &g, long long off,
                                                const NbrRec *__restrict__ nbr,
                                                const CullRec *__restrict__ cull,
                                                const int *__restrict__ start,
                                                const int *__restrict__ order, unsigned want, V3 &F,
                                                V3 &T) {
  const bool xi0 = c.variant == AF3D_FRICTION_DEV;
  const CullRec me = cull[s];
  const Search q = search_centre(o.r, g, off);
  int active = 0;
#pragma unroll 1
  for (int p = 0; p < 16; p++) {
    if (!((want >> p) & 1u)) continue;
    const int sl = p & 3, sm = p >> 2;
    for_neighbour_slots(q, g, start, order, [&](int t) {
      if (t == s) return;
      if (!((pair_mask(me, cull[t]) >> p) & 1u)) return;
      active += part_pair(o.r, o.v, o.w, o.s[sl], o.rad, o.msph, nbr[t], sm, c, xi0, F, T) == 2;
    });
  }
  return active;
}

// Per-clump contact pass (one thread, its own item list): the per-routine force_part entry.
__device__ __forceinline__ int particle_contacts(long s, const Own &o, const Consts &c,
                                                 const af3d_cell_par &g, long long off,
                                                 const NbrRec *__restrict__ nbr,
                                                 const CullRec *__restrict__ cull,
                                                 const int *__restrict__ start,
                                                 const int *__restrict__ order, int only_p, V3 &F,
                                                 V3 &T) {
  const bool xi0 = c.variant == AF3D_FRICTION_DEV;
  const unsigned want = only_p < 0 ? 0xffffu : (1u << only_p);
  unsigned items[kItemCap];
  int nitems = 0;
  if (!gather_items(s, o, g, off, cull, start, order, want, items, kItemCap, nitems))
    return contacts_by_pass(s, o, c, g, off, nbr, cull, start, order, want, F, T);
  int active = 0;
#pragma unroll 1
  for (int i = 0; i < nitems; i++) {
    const int t = (int)(items[i] >> 4), p = (int)(items[i] & 15u);
    active += part_pair(o.r, o.v, o.w, o.s[p & 3], o.rad, o.msph, nbr[t], p >> 2, c, xi0, F, T) == 2;
  }
  return active;
}

// Block-cooperative pass of the fused kernel over every contact of a clump: the boundary routines
// that run before the particle contacts, the sixteen sph_id passes, and the routines that run
// after them (avalanche: hop x3, funnel, fcorners, walls | part x16 | flume; fill: part x16 |
// hop x3).  The list phase (lists_body) has published every clump's item list in that
// order: boundary items (routine, sphere) for the spheres the routine's 1-Lipschitz gate cannot
// rule out, and particle items (partner slot, sph_id) of overlapping sphere pairs in sph_id-major
// order.  The block concatenates the lists of its clumps and works through them in batches of
// kBatch items, 32 items a round per warp, one item per lane, reading the owner clump from its
// record; after each batch every owner adds its items' force and torque terms to its own sums in
// list order.  The FP64 contact laws thus run with nearly all lanes busy whatever the spread of
// contacts and walls over the clumps, and each clump's summation order stays the reference's.
// Every thread of the block must call this; `act` is false for threads without a clump to
// process (and for removed clumps).  A clump whose lists overflowed runs alone afterwards, in
// the same order.
constexpr int kBatch = 256;
template <int NB>
struct BlockQueue {
  int base[NB + 1];   // exclusive prefix of the clumps' item counts
  int pbase[NB + 1];  // ... of their particle item counts (kind-sorted pass)
  int qbase[NB + 1];  // ... of their boundary item counts (kind-sorted pass)
  int npre[NB];       // boundary items before the particle items, per clump
  int wsum[3][NB / 32];
  double res[6][kBatch];  // [component][item in the batch]
  unsigned char flag[kBatch];
};

// The thread whose range [base[t], base[t+1]) holds position j.
template <int NB>
__device__ __forceinline__ int block_owner_of(const int *base, int j) {
  int lo = 0, hi = NB - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Block-wide exclusive prefixes of three per-thread counts (all threads call this).
template <int NB>
__device__ __forceinline__ void block_prefix3(BlockQueue<NB> &bq, int a, int b, int c) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int v[3] = {a, b, c};
#pragma unroll
  for (int q = 0; q < 3; q++) {
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v[q], k);
      if (lane >= k) v[q] += u;
    }
    if (lane == 31) bq.wsum[q][warp] = v[q];
  }
  __syncthreads();
  int *dst[3] = {bq.base, bq.pbase, bq.qbase};
  const int own[3] = {a, b, c};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    int wofs = 0, total = 0;
#pragma unroll
    for (int w = 0; w < NB / 32; w++) {
      const int t = bq.wsum[q][w];
      wofs += w < warp ? t : 0;
      total += t;
    }
    dst[q][tid] = wofs + v[q] - own[q];
    if (tid == NB - 1) dst[q][NB] = total;
  }
  __syncthreads();
}

__device__ __forceinline__ Own own_from_record(const NbrRec &q) {
  Own o;
  o.r = mk(q.rx, q.ry, q.rz);
  o.v = mk(q.vx, q.vy, q.vz);
  o.w = mk(q.wx, q.wy, q.wz);
  for (int k = 0; k < 4; k++) o.s[k] = mk(q.s[3 * k], q.s[3 * k + 1], q.s[3 * k + 2]);
  o.rad = q.rad;
  o.msph = q.msph;
  o.mwall = q.mwall;
  return o;
}

__device__ __forceinline__ Own own_from_planes(const Planes &P, long s) {
  Own o;
  o.r = load3(P, RX, s);
  o.v = load3(P, VX, s);
  o.w = load3(P, WX, s);
  for (int k = 0; k < 4; k++) o.s[k] = load3(P, S0X + 3 * k, s);
  o.rad = P.p[RAD][s];
  o.msph = P.p[MSPH][s];
  o.mwall = P.p[MWALL][s];
  return o;
}

// The contacts of a clump whose item lists overflowed, by the per-clump cell walk, added to
// (F, T) in the reference's order: the boundary routines before the particles, the sixteen
// sph_id passes, the routines after.  Not inlined: it runs rarely, and inlined its registers
// and spills would weigh on the pooled path of every clump.  The clump's state, bound and
// grid are read here again.
struct SlowSums {
  V3 F, T;
  int active;
};
__device__ __noinline__ SlowSums slow_contacts(long s, int pre0, int pre1, int post0, int post1, const Consts &c,
                                               const DevScalars *d, const int *__restrict__ flume,
                                               const NbrRec *__restrict__ nbr, const CullRec *__restrict__ cull,
                                               const int *__restrict__ start, const int *__restrict__ order, V3 F,
                                               V3 T) {
  const Own o = own_from_record(nbr[s]);
  const double B = (double)cull[s].c.w;
  const DevFlume &fl = d->flumes[flume[s]];
  for (int rt = pre0; rt <= pre1; rt++)
    if (bnd_may_touch(rt, o.r, B, c)) bnd_routine(rt, o, false, c, F, T);
  const int active = contacts_by_pass(s, o, c, fl.grid, fl.cell_off, nbr, cull, start, order, 0xffffu, F, T);
  for (int rt = post0; rt <= post1; rt++)
    if (bnd_may_touch(rt, o.r, B, c)) bnd_routine(rt, o, false, c, F, T);
  return SlowSums{F, T, active};
}

// A boundary item's contact, prepared for the law.  Not inlined: the seven routines' input code
// inlined into the pooled item loop raised its register pressure enough to spill on every
// clump's path (636 bytes of spill stores against 212), while boundary items are a minority of
// the items.
__device__ __noinline__ bool bnd_input_call(int rt, const Sph &q, const Consts &co, ContactIn &ci) {
  return bnd_input(rt, q, co, ci);
}

// UNIFORM: every clump of the launch belongs to one flume, whose constants `c` are (a
// reference to) a kernel parameter.  lc: the clump's list layout (pre boundary items, particle
// items, the rest boundary items).
template <int NB, bool UNIFORM>
__device__ __forceinline__ int block_contacts(BlockQueue<NB> &bq, long bbase, long s, bool act, bool aval,
                                              const Consts &c, const DevScalars *d, const int *__restrict__ flume,
                                              const NbrRec *__restrict__ nbr,
                                              const CullRec *__restrict__ cull,
                                              const int *__restrict__ start,
                                              const int *__restrict__ order,
                                              const unsigned *items, int listed, ListCounts lc, long n,
                                              V3 &F, V3 &T) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int pre0 = aval ? R_HOP0 : 1, pre1 = aval ? R_WALLS : 0;         // fill: none before
  const int post0 = aval ? R_FLUME : R_HOP0, post1 = aval ? R_FLUME : R_HOP2;
  const bool slow = act && listed < 0;
  const int nitems = act && listed > 0 ? listed : 0;
  const int npair = nitems > 0 ? lc.pair : 0;
  bq.npre[tid] = nitems > 0 ? lc.pre : 0;
  block_prefix3<NB>(bq, nitems, npair, nitems - npair);
  const int base = bq.base[tid], total = bq.base[NB];
  const int ptotal = bq.pbase[NB];
  // One item: its contact into the batch's result slot jb.
  auto process = [&](int lo, int idx, int jb) {
    const unsigned it = items[(long)idx * n + bbase + lo];   // written in this launch
    const NbrRec &me = nbr[bbase + lo];   // owners hold clumps, so bbase + lo < n
    // Prepare the item's contact (type-specific, short), then run the contact law.
    auto contact = [&](const Consts &co, V3 &fs, V3 &tq) -> int {
      ContactIn ci;
      V3 rl = mk(me.rx, me.ry, me.rz);
      int kind;   // 0 nothing, 1 sphere pair, 2 wall
      if (it >= kBndItem) {
        const int rt = (int)((it >> 2) & 7u), ns = (int)(it & 3u);
        Sph q;
        q.r = rl;
        q.v = mk(me.vx, me.vy, me.vz);
        q.w = mk(me.wx, me.wy, me.wz);
        q.s = mk(me.s[3 * ns], me.s[3 * ns + 1], me.s[3 * ns + 2]);
        q.rad = me.rad;
        q.mwall = me.mwall;
        kind = bnd_input_call(rt, q, co, ci) ? 2 : 0;
      } else {
        const int t = (int)(it >> 4), p = (int)(it & 15u);
        const V3 vl = mk(me.vx, me.vy, me.vz), wl = mk(me.wx, me.wy, me.wz);
        const int k = p & 3;
        const V3 s1 = mk(me.s[3 * k], me.s[3 * k + 1], me.s[3 * k + 2]);
        kind = pair_input(rl, vl, wl, s1, me.rad, me.msph, nbr[t], p >> 2, co,
                          co.variant == AF3D_FRICTION_DEV, ci, true) ? 1 : 0;
      }
      int r = kind == 1 ? 1 : 0;
      if (kind && apply_law(ci, rl, co, fs, tq)) r = kind == 1 ? 2 : 3;
      return r;
    };
    V3 fs, tq;
    int r;
    if constexpr (UNIFORM) {
      r = contact(c, fs, tq);
    } else {
      // the owner's flume may differ from this thread's at a flume boundary of an ensemble
      const int of = flume[bbase + lo];
      const Consts &co = of == flume[s] ? c : d->flumes[of].c;
      r = contact(co, fs, tq);
    }
    bq.flag[jb] = (unsigned char)r;
    if (r >= 2) {
      bq.res[0][jb] = fs.x; bq.res[1][jb] = fs.y; bq.res[2][jb] = fs.z;
      bq.res[3][jb] = tq.x; bq.res[4][jb] = tq.y; bq.res[5][jb] = tq.z;
    }
  };
  int active = 0;
  // Owners add their items' terms in list order.
  auto gather = [&](int b0, int bn) {
    if (nitems <= 0) return;
    const int a = base > b0 ? base : b0;
    const int b = base + nitems < b0 + bn ? base + nitems : b0 + bn;
    for (int e = a - b0; e < b - b0; e++) {
      const int fl = bq.flag[e];
      if (fl < 2) continue;
      T.x += bq.res[3][e]; T.y += bq.res[4][e]; T.z += bq.res[5][e];
      F.x += bq.res[0][e]; F.y += bq.res[1][e]; F.z += bq.res[2][e];
      active += fl == 2;   // sphere-sphere contacts only
    }
  };
  // A block whose items fit one batch takes them in kind order: every particle item of the
  // block, then every boundary item, 32 a round per warp, so that each round runs one input
  // routine; results go to the items' places in the owners' lists.  Otherwise batches of kBatch
  // items in the owners' order.
  const bool kind_order = total <= kBatch;
  for (int b0 = 0; b0 < total; b0 += kBatch) {
    const int bn = total - b0 < kBatch ? total - b0 : kBatch;
    for (int r0 = warp * 32; r0 < bn; r0 += NB) {
      const int i = r0 + lane;
      if (i < bn) {
        int lo, idx;
        if (kind_order && i < ptotal) {
          lo = block_owner_of<NB>(bq.pbase, i);
          idx = bq.npre[lo] + (i - bq.pbase[lo]);
        } else if (kind_order) {
          const int ib = i - ptotal;
          lo = block_owner_of<NB>(bq.qbase, ib);
          const int b = ib - bq.qbase[lo], np = bq.npre[lo];
          idx = b < np ? b : b + (bq.pbase[lo + 1] - bq.pbase[lo]);
        } else {
          lo = block_owner_of<NB>(bq.base, b0 + i);   // the thread whose list holds item b0 + i
          idx = b0 + i - bq.base[lo];
        }
        process(lo, idx, kind_order ? bq.base[lo] + idx : i);
      }
    }
    __syncthreads();
    gather(b0, bn);
    __syncthreads();
  }
  if (slow) {
    const SlowSums r = slow_contacts(s, pre0, pre1, post0, post1, c, d, flume, nbr, cull, start, order, F, T);
    F = r.F;
    T = r.T;
    active += r.active;
  }
  return active;
}

__device__ __forceinline__ void warp_count(DevScalars *d, int active) {
  unsigned v = (unsigned)active;
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&d->contacts, (unsigned long long)v);
}

// The list phase of k_lists_forces for one clump: its item lists (see block_contacts) into
// `lists`; returns the item count (-1: the lists overflowed) and their layout in lc.
template <bool UNIFORM>
__device__ __forceinline__ int lists_body(const Consts &c, const DevScalars *d, const int *__restrict__ flume,
                                           const NbrRec *__restrict__ nbr, const CullRec *__restrict__ cull,
                                           const int *__restrict__ start, const int *__restrict__ order,
                                           const float4 *__restrict__ csort, ContactLists lists, long s0,
                                           long n, PassLists &pl, ListCounts &lc) {
  const long s = s0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = s < n;
  const long sv = valid ? s : n - 1;
  const int f = flume[sv];
  const DevFlume &fl = d->flumes[f];
  const af3d_cell_par g = fl.grid;
  const GridF gf = fl.gridf;
  const long long off = fl.cell_off;
  const NbrRec &me = nbr[sv];
  const V3 r = mk(me.rx, me.ry, me.rz);
  const bool act = valid && !is_removed(*c.tp, r.x, c.side_x);
  bool slow = false;
  const int k = build_item_lists(pl, lists.items + sv, n, s0 + blockIdx.x * (long)blockDim.x + (threadIdx.x & ~31u), sv,
                                 act, c.phase == AF3D_PHASE_AVALANCHE, r, c, g, gf, off, nbr, cull, start, order,
                                 csort, slow, lc);
  return slow ? -1 : k;
}

// Shared memory of the force kernel: the list phase, the force phase and the look-ahead's record
// staging run one after another.  Kept small because the SM's L1 cache gets what the resident
// blocks' shared memory leaves of 256 KB: at 96 threads and 6 blocks an SM, 20.3 KB per block
// (the list phase's) leaves ~124 KB of L1 for the walk's, records' and spills' lines, where
// 30.8 KB left 60 KB (0.275 -> 0.269 ms per pass on the 262,144-clump bed).
template <int NB>
union ForceShared {
  PassLists pl[NB / 32];
  BlockQueue<NB> bq;
  struct {
    double nbr[NB * kRecStride];
  } rec;
};

template <int NB, bool WRITE_FT, bool UNIFORM>
__device__ __forceinline__ void fused_body(const Consts &c, Planes P, Planes out, DevScalars *d,
                                           const int *__restrict__ flume, const NbrRec *__restrict__ nbr,
                                           const CullRec *__restrict__ cull, const int *__restrict__ start,
                                           const int *__restrict__ order, ContactLists lists, int listed,
                                           ListCounts lc, long s0, long n, bool warm, const LookAhead &la,
                                           ForceShared<NB> &sh) {
  const long s = s0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = s < n;
  const long sv = valid ? s : n - 1;   // in-range slot for lanes past n (nothing is written for them)
  const int f = flume[sv];
  const bool removed = is_removed(*c.tp, nbr[sv].rx, c.side_x);
  V3 F = mk(0.0, 0.0, 0.0), T = mk(0.0, 0.0, 0.0);
  const bool aval = c.phase == AF3D_PHASE_AVALANCHE;
  // Removed clumps get hop, funnel and fcorners only (walls, part and flume skip them).
  if (valid && removed && aval) {
    const Own o = own_from_record(nbr[sv]);
    const double B = (double)cull[sv].c.w;   // sphere offsets + radius, rounded up
    for (int rt = R_HOP0; rt <= R_FCORNERS; rt++)
      if (bnd_may_touch(rt, o.r, B, c)) bnd_routine(rt, o, true, c, F, T);
  }
  const long bbase = s0 + blockIdx.x * (long)blockDim.x;
  const int active = block_contacts<NB, UNIFORM>(sh.bq, bbase, sv, valid && !removed, aval, c, d, flume, nbr, cull,
                                                 start, order, lists.items, valid ? listed : 0, lc, n, F, T);
  if (la.nbr) __syncthreads();   // the force phase's shared memory is free for the record staging
  if (valid) {
    if (lists.cnt) lists.cnt[s] = pack_list_counts(listed, lc.pre, lc.pair);
    if (lists.ovf && listed < 0) *lists.ovf = 1;
    if (listed < 0) atomicAdd(&d->overflows, 1ull);   // rare: counted for the diagnostics
    if (WRITE_FT) {
      store3(P, FX, s, F);
      store3(P, TX, s, T);
    }
    // this step's predicted state, read again from the record (not held across the contacts);
    // its rotation rows from the RN planes when the previous pass predicted it
    const NbrRec &me = nbr[s];
    const V3 r = mk(me.rx, me.ry, me.rz);
    const V3 v = mk(me.vx, me.vy, me.vz), w = mk(me.wx, me.wy, me.wz);
    const int R0 = warm ? RN00 : R00;
    V3 Rx = load3(P, R0, s), Ry = load3(P, R0 + 3, s), Rz = load3(P, R0 + 6, s);
    if (warm) {   // commit the predicted state to the planes
      store3(P, RX, s, r);
      for (int k = 0; k < 4; k++) store3(P, S0X + 3 * k, s, mk(me.s[3 * k], me.s[3 * k + 1], me.s[3 * k + 2]));
      store3(P, R00, s, Rx);
      store3(P, R10, s, Ry);
      store3(P, R20, s, Rz);
    }
    V3 v2, w2, a, al;
    if (!removed) {
      get_accel_one(F, T, v, w, Rx, Ry, Rz, P.p[MASS][s], P.p[ADRAG][s], load3(P, IXX, s), a, al, P.p[IMASS][s],
                    P.p[IINER][s]);
      store3(P, AFX, s, a);
      store3(P, ALFX, s, al);
      const V3 ai = load3(P, AIX, s), ali = load3(P, ALIX, s);
      // finish_Verlet.cu:43-48
      v2 = mk(v.x + c.hdt * (a.x - ai.x), v.y + c.hdt * (a.y - ai.y), v.z + c.hdt * (a.z - ai.z));
      w2 = mk(w.x + c.hdt * (al.x - ali.x), w.y + c.hdt * (al.y - ali.y), w.z + c.hdt * (al.z - ali.z));
      if (!(finite_bits(a.x) && finite_bits(a.y) && finite_bits(a.z) && finite_bits(al.x) && finite_bits(al.y) &&
            finite_bits(al.z)))
        raise_status(d, AF3D_ERR_NAN);
    } else {
      v2 = mk(0.0, 0.0, 0.0);                 // finish_Verlet.cu:28-32
      w2 = w;
      a = al = mk(0.0, 0.0, 0.0);             // the reference leaves stale values here
      store3(P, AFX, s, a);
      store3(P, ALFX, s, al);
    }
    store3(out, VX, s, v2);
    store3(out, WX, s, w2);
    if (la.nbr) {
      // The next step's init_Verlet (removal test at this step's time, a_i = this a_f), cell key
      // (at the next step's time) and records, exactly as k_predict<1,1,1> would make them
      // after this step.
      const DevFlume &fl = d->flumes[f];
      const double t_next = *c.tp + d->flumes[0].sys.dt;   // k_advance_time's expression
      V3 rn = r, vn = v2, wn = w2, sp[4];
      if (is_removed(*c.tp, r.x, fl.sys.side.x)) {
        P.p[RAD][s] = 0.0;
        for (int k = 0; k < 4; k++) sp[k] = mk(me.s[3 * k], me.s[3 * k + 1], me.s[3 * k + 2]);
        store3(P, RN00, s, Rx);
        store3(P, RN10, s, Ry);
        store3(P, RN20, s, Rz);
      } else {
        predict_state(rn, vn, wn, a, al, Rx, Ry, Rz, sp, P.p[RAD][s], fl.sys.dt, fl.sys.hdt);
        store3(P, RN00, s, Rx);
        store3(P, RN10, s, Ry);
        store3(P, RN20, s, Rz);
      }
      {
        NbrRec q;
        CullRec cr;
        make_records(rn, vn, wn, sp, P.p[RAD][s], P.p[MSPH][s], P.p[MWALL][s], q, cr);
        stage_nbr_record(q, sh.rec.nbr);
        la.cull[s] = cr;   // stored directly: staged too, it would set the block's shared memory size
      }
      const long key = bucket_key(rn, fl, d, la.id[s], t_next);
      la.cells.key[s] = (int)key;
      la.cells.rank_tmp[s] = arrive_in_bucket(la.cells, key);
    }
  }
  warp_count(d, active);
  if (la.nbr) {
    __syncthreads();   // every neighbour record of the block is staged
    copy_nbr_records<NB>(bbase, n, la.nbr, sh.rec.nbr);
  }
}

// One boundary routine added to the F, T planes (per-routine entry points).
__global__ void k_boundary(Planes P, DevScalars *d, const int *__restrict__ flume, int routine, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const Consts c = load_consts(d, flume[s]);
  const Own o = own_from_planes(P, s);
  const bool removed = is_removed(*c.tp, o.r.x, c.side_x);
  V3 F = load3(P, FX, s), T = load3(P, TX, s);
  bnd_routine(routine, o, removed, c, F, T);
  store3(P, FX, s, F);
  store3(P, TX, s, T);
}

// force_part for one sph_id (1..16) or all sixteen (0), added to the F, T planes.
__global__ void __launch_bounds__(kBlock) k_part(Planes P, DevScalars *d, const int *__restrict__ flume,
                                                 const NbrRec *__restrict__ nbr,
                                                 const CullRec *__restrict__ cull,
                                                 const int *__restrict__ start, int sph_id, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int f = flume[s];
  const Consts c = load_consts(d, f);
  const af3d_cell_par g = d->flumes[f].grid;
  const Own o = own_from_planes(P, s);
  if (is_removed(*c.tp, o.r.x, c.side_x)) return;
  V3 F = load3(P, FX, s), T = load3(P, TX, s);
  particle_contacts(s, o, c, g, d->flumes[f].cell_off, nbr, cull, start, nullptr, sph_id - 1, F, T);
  store3(P, FX, s, F);
  store3(P, TX, s, T);
}

__global__ void k_get_accel(Planes P, DevScalars *d, const int *__restrict__ flume, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  if (is_removed(d->time, P.p[RX][s], d->flumes[flume[s]].sys.side.x)) return;
  V3 a, al;
  get_accel_one(load3(P, FX, s), load3(P, TX, s), load3(P, VX, s), load3(P, WX, s), load3(P, R00, s),
                load3(P, R10, s), load3(P, R20, s), P.p[MASS][s], P.p[ADRAG][s], load3(P, IXX, s), a, al, P.p[IMASS][s], P.p[IINER][s]);
  store3(P, AFX, s, a);
  store3(P, ALFX, s, al);
}

__global__ void k_finish_verlet(Planes P, DevScalars *d, const int *__restrict__ flume, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const af3d_system_par &sy = d->flumes[flume[s]].sys;
  const double hdt = sy.hdt;
  if (is_removed(d->time, P.p[RX][s], sy.side.x)) {
    store3(P, VX, s, mk(0.0, 0.0, 0.0));
    return;
  }
  V3 v = load3(P, VX, s), w = load3(P, WX, s);
  V3 af = load3(P, AFX, s), ai = load3(P, AIX, s), alf = load3(P, ALFX, s), ali = load3(P, ALIX, s);
  v.x += hdt * (af.x - ai.x);
  v.y += hdt * (af.y - ai.y);
  v.z += hdt * (af.z - ai.z);
  w.x += hdt * (alf.x - ali.x);
  w.y += hdt * (alf.y - ali.y);
  w.z += hdt * (alf.z - ali.z);
  store3(P, VX, s, v);
  store3(P, WX, s, w);
}

__global__ void k_clear_forces(Planes P, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  store3(P, FX, s, mk(0.0, 0.0, 0.0));
  store3(P, TX, s, mk(0.0, 0.0, 0.0));
}

// sys_par.time += dt (avalanche_hst.cu:672), keeping the previous value for init_Verlet.  The
// flumes of an ensemble share dt and the clock.
__global__ void k_advance_time(DevScalars *d) {
  d->time_prev = d->time;
  d->time = d->time + d->flumes[0].sys.dt;
}

// ------------------------------------------------------------------ re-grid (cell_dim)

__device__ __forceinline__ unsigned long long ord(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

__global__ void k_bbox_init(DevScalars *d, int nflumes) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nflumes) return;
  unsigned long long *b = d->flumes[f].bbox;
  for (int i = 0; i < 3; i++) {
    b[i] = ~0ull;    // min x, y, z
    b[3 + i] = 0ull; // max x, y, z
  }
  b[6] = 0ull;       // max vx
  b[7] = ~0ull;      // min vz
}

// Min/max of clump centres, max vx and min vz over every clump of each flume (cell_dim.cu:21-54),
// warp-reduced when a warp's clumps belong to one flume.
__global__ void k_bbox_reduce(Planes P, DevScalars *d, const int *__restrict__ flume, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long sv = s < n ? s : n - 1;
  const int f = flume[sv];
  unsigned long long mn[3], mx[3], vx, vz;
  for (int i = 0; i < 3; i++) mn[i] = mx[i] = ord(P.p[RX + i][sv]);
  vx = ord(P.p[VX][sv]);
  vz = ord(P.p[VZ][sv]);
  const int f0 = __shfl_sync(0xffffffffu, f, 0);
  const bool uniform = __all_sync(0xffffffffu, f == f0);
  if (uniform) {
    for (int off = 16; off; off >>= 1) {
      for (int i = 0; i < 3; i++) {
        mn[i] = min(mn[i], __shfl_xor_sync(0xffffffffu, mn[i], off));
        mx[i] = max(mx[i], __shfl_xor_sync(0xffffffffu, mx[i], off));
      }
      vx = max(vx, __shfl_xor_sync(0xffffffffu, vx, off));
      vz = min(vz, __shfl_xor_sync(0xffffffffu, vz, off));
    }
  }
  if (!uniform || (threadIdx.x & 31) == 0) {
    unsigned long long *b = d->flumes[f].bbox;
    for (int i = 0; i < 3; i++) {
      atomicMin(&b[i], mn[i]);
      atomicMax(&b[3 + i], mx[i]);
    }
    atomicMax(&b[6], vx);
    atomicMin(&b[7], vz);
  }
}

// cell_dim.cu:56-66 padding and the grid derivation of avalanche_hst.cu:314-333, per flume, into
// the flume's pending grid.
__global__ void k_grid_derive(DevScalars *d, int nflumes) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nflumes) return;
  DevFlume &fl = d->flumes[f];
  if (fl.bbox[0] == ~0ull) {
    // A flume without clumps keeps its grid (a one-cell grid if it never had one): nothing is
    // binned there, and cell_dim would read a clump that does not exist.
    af3d_cell_par g = fl.grid;
    if (g.ncell3 <= 0) {
      g.rr_min = {0.0, 0.0, 0.0};
      g.rr_max = g.length = g.cell_side = g.cs_inv = {1.0, 1.0, 1.0};
      g.ncell = {1, 1, 1};
      g.ncell3 = 1;
      g.ntot = g.ntags;
    }
    fl.pending = g;
    return;
  }
  const af3d_system_par &sy = fl.sys;
  const double rgyr = 0.5 * sy.gyr_max, ddt = 2000.0 * sy.dt;
  const double vxmax = unord(fl.bbox[6]), vzmin = unord(fl.bbox[7]);
  V3 hi = mk(unord(fl.bbox[3]), unord(fl.bbox[4]), unord(fl.bbox[5]));
  V3 lo = mk(unord(fl.bbox[0]), unord(fl.bbox[1]), unord(fl.bbox[2]));
  hi.x += 1.05 * rgyr + vxmax * ddt;
  lo.x -= 1.05 * rgyr;
  hi.y += 1.05 * rgyr;
  lo.y -= 1.05 * rgyr;
  hi.z += 1.05 * rgyr;
  lo.z -= 1.05 * rgyr - vzmin * ddt;
  af3d_cell_par g = fl.grid;
  const double dist = kGYR + (double)0.05f;   // avalanche_hst.cu:115 adds a float literal
  g.rr_max = {hi.x, hi.y, hi.z};
  g.rr_min = {lo.x, lo.y, lo.z};
  g.length = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
  g.ncell.x = (long)(g.length.x / (dist * sy.rmax));
  g.ncell.y = (long)(g.length.y / (dist * sy.rmax));
  g.ncell.z = (long)(g.length.z / (dist * sy.rmax));
  g.cell_side.x = g.length.x / ((double)g.ncell.x);
  g.cell_side.y = g.length.y / ((double)g.ncell.y);
  g.cell_side.z = g.length.z / ((double)g.ncell.z);
  g.cs_inv.x = 1.0 / g.cell_side.x;
  g.cs_inv.y = 1.0 / g.cell_side.y;
  g.cs_inv.z = 1.0 / g.cell_side.z;
  g.ncell3 = g.ncell.x * g.ncell.y * g.ncell.z;
  g.ntot = g.ncell3 * g.ntags;
  fl.pending = g;
}

// Commit the pending grids with their bucket offsets when every grid is non-empty and the
// buckets fit; otherwise record the buckets needed (-1: an empty grid) and keep the old grids.
__global__ void k_grid_commit(DevScalars *d, int nflumes, long n, long bucket_cap) {
  long long total = 0;
  bool ok = true;
  for (int f = 0; f < nflumes; f++) {
    const long long c = d->flumes[f].pending.ncell3;
    ok = ok && c > 0;
    total += c > 0 ? c : 0;
  }
  if (!ok) {
    d->pending = -1;
    return;
  }
  if (total + n + 1 > bucket_cap) {
    d->pending = total;
    return;
  }
  long long off = 0;
  for (int f = 0; f < nflumes; f++) {
    d->flumes[f].grid = d->flumes[f].pending;
    d->flumes[f].gridf = grid_floats(d->flumes[f].grid);
    d->flumes[f].cell_off = off;
    off += d->flumes[f].grid.ncell3;
  }
  d->ncell_total = total;
  d->pending = 0;
}

// ------------------------------------------------------------------ diagnostics

__global__ void k_contact_pairs(Planes P, DevScalars *d, const int *__restrict__ flume,
                                const NbrRec *__restrict__ nbr, const CullRec *__restrict__ cull,
                                const int *__restrict__ start, const long long *__restrict__ id,
                                long long *out, unsigned long long *count, long cap, int active_only,
                                long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int f = flume[s];
  const Consts c = load_consts(d, f);
  const af3d_cell_par g = d->flumes[f].grid;
  const Own o = own_from_planes(P, s);
  if (is_removed(*c.tp, o.r.x, c.side_x)) return;
  const CullRec me = cull[s];
  const Search q = search_centre(o.r, g, d->flumes[f].cell_off);
  for_neighbour_slots(q, g, start, nullptr, [&](int t) {
    if (t == s) return;
    unsigned m = pair_mask(me, cull[t]);
    while (m) {
      const int p = __ffs(m) - 1;
      m &= m - 1;
      V3 F = mk(0.0, 0.0, 0.0), T = mk(0.0, 0.0, 0.0);
      const int r = part_pair(o.r, o.v, o.w, o.s[p & 3], o.rad, o.msph, nbr[t], p >> 2, c, false, F, T);
      if (r == 2 || (r == 1 && !active_only)) {
        unsigned long long k = atomicAdd(count, 1ull);
        if ((long)k < cap) {
          out[3 * k] = id[s];
          out[3 * k + 1] = id[t];
          out[3 * k + 2] = p + 1;
        }
      }
    }
  });
}

// Bucket of every clump by id (-1 when not binned): the flume's cell offset plus the cell index.
__global__ void k_cells_by_id(const int *__restrict__ key, const long long *__restrict__ id,
                              const DevScalars *d, long long *cell_of_id, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int k = key[s];
  cell_of_id[id[s]] = k < d->ncell_total ? k : -1;
}

}  // namespace

// ------------------------------------------------------------------ launchers

// Built twice: the exact launchers in namespace af3d, and (with -DAF3D_FAST) the fast-mode
// build of the same kernels, whose predictor and force launchers the context uses in fast mode.
#ifdef AF3D_FAST
namespace fast {
#endif

void launch_predict(const Launch &L, Planes cur, DevScalars *d, bool predict, bool keys, bool t_prev,
                    Cells cells, const long long *id, const int *flume, NbrRec *nbr, CullRec *cull, long s0,
                    long count) {
  // slots [s0, s0 + count) of L.n (count < 0: to the end); s0 a multiple of kBlock
  const long m = count < 0 ? L.n - s0 : std::min(count, L.n - s0);
  if (L.n <= 0 || m <= 0 || s0 % kBlock != 0) return;
  const unsigned g = grid_for(m);
  if (predict && keys && nbr)
    k_predict<true, true, true><<<g, kBlock, 0, L.st>>>(cur, d, t_prev, cells, id, flume, nbr, cull, s0, L.n);
  else if (predict && keys)
    k_predict<true, true, false><<<g, kBlock, 0, L.st>>>(cur, d, t_prev, cells, id, flume, nbr, cull, s0, L.n);
  else if (predict)
    k_predict<true, false, false><<<g, kBlock, 0, L.st>>>(cur, d, t_prev, cells, id, flume, nbr, cull, s0, L.n);
  else if (keys && nbr)
    k_predict<false, true, true><<<g, kBlock, 0, L.st>>>(cur, d, t_prev, cells, id, flume, nbr, cull, s0, L.n);
  else if (keys)
    k_predict<false, true, false><<<g, kBlock, 0, L.st>>>(cur, d, t_prev, cells, id, flume, nbr, cull, s0, L.n);
}

void launch_permute_records(const Launch &L, Planes src, Planes dst, const int *perm,
                            const long long *id_src, long long *id_dst, const int *fl_src, int *fl_dst,
                            NbrRec *nbr, CullRec *cull, bool ft) {
  if (L.n <= 0) return;
  k_permute<<<grid_for(L.n, kPermBlock), kPermBlock, 0, L.st>>>(src, dst, perm, id_src, id_dst, fl_src,
                                                                fl_dst, nbr, cull, ft, L.n);
}

void launch_build_records(const Launch &L, Planes cur, NbrRec *nbr, CullRec *cull) {
  if (L.n <= 0) return;
  k_permute<<<grid_for(L.n, kPermBlock), kPermBlock, 0, L.st>>>(cur, cur, nullptr, nullptr, nullptr,
                                                                nullptr, nullptr, nbr, cull, true, L.n);
}

// The lists and the force pass of one block's clumps in one launch: the block builds its clumps'
// item lists (the list kernel's work), then processes them (the force kernel's work).  Blocks
// resident on one SM are in different phases most of the time, so the latency-bound walk of
// some overlaps the FP64-bound contact laws of others.  The lists pass through global memory
// (the block's own entries, visible to its threads after the barrier).
template <int NB, int MINB, bool WRITE_FT, bool UNIFORM>
__global__ void __launch_bounds__(NB, MINB) k_lists_forces(Planes P, Planes out, DevScalars *d,
                                                         const int *__restrict__ flume,
                                                         const NbrRec *__restrict__ nbr,
                                                         const CullRec *__restrict__ cull,
                                                         const int *__restrict__ start,
                                                         const int *__restrict__ order,
                                                         const float4 *__restrict__ csort, ContactLists lists,
                                                         const __grid_constant__ Consts kc, bool warm,
                                                         const __grid_constant__ LookAhead la, long s0, long n) {
  __shared__ ForceShared<NB> sh;
  ListCounts lc;
  if constexpr (UNIFORM) {
    const int listed = lists_body<true>(kc, d, flume, nbr, cull, start, order, csort, lists, s0, n,
                                        sh.pl[threadIdx.x >> 5], lc);
    __syncthreads();
    fused_body<NB, WRITE_FT, true>(kc, P, out, d, flume, nbr, cull, start, order, lists, listed, lc, s0, n, warm, la,
                               sh);
  } else {
    // the flume's constants read where they lie (a reference, not a register copy)
    const long s = s0 + blockIdx.x * (long)blockDim.x + threadIdx.x;
    const Consts &c = d->flumes[flume[s < n ? s : n - 1]].c;
    const int listed = lists_body<false>(c, d, flume, nbr, cull, start, order, csort, lists, s0, n,
                                         sh.pl[threadIdx.x >> 5], lc);
    __syncthreads();
    fused_body<NB, WRITE_FT, false>(c, P, out, d, flume, nbr, cull, start, order, lists, listed, lc, s0, n, warm, la,
                                sh);
  }
}

template <int NB, int MINB>
void launch_lists_forces_shape(const Launch &L, Planes cur, Planes out, DevScalars *d, const int *flume,
                               const NbrRec *nbr, const CullRec *cull, const int *start, const int *order,
                               const float4 *csort, ContactLists lists, bool write_ft, const Consts *uniform,
                               bool warm, LookAhead look, long s0, long m) {
  const Consts kc = uniform ? *uniform : Consts{};
  const unsigned g = grid_for(m, NB);
  if (uniform) {
    if (write_ft)
      k_lists_forces<NB, MINB, true, true><<<g, NB, 0, L.st>>>(cur, out, d, flume, nbr, cull, start, order, csort,
                                                              lists, kc, warm, look, s0, L.n);
    else
      k_lists_forces<NB, MINB, false, true><<<g, NB, 0, L.st>>>(cur, out, d, flume, nbr, cull, start, order, csort,
                                                               lists, kc, warm, look, s0, L.n);
  } else {
    if (write_ft)
      k_lists_forces<NB, MINB, true, false><<<g, NB, 0, L.st>>>(cur, out, d, flume, nbr, cull, start, order, csort,
                                                               lists, kc, warm, look, s0, L.n);
    else
      k_lists_forces<NB, MINB, false, false><<<g, NB, 0, L.st>>>(cur, out, d, flume, nbr, cull, start, order, csort,
                                                                lists, kc, warm, look, s0, L.n);
  }
}

void launch_lists_forces(const Launch &L, Planes cur, Planes out, DevScalars *d, const int *flume,
                         const NbrRec *nbr, const CullRec *cull, const int *start, const int *order,
                         const float4 *csort, ContactLists lists, bool write_ft, const Consts *uniform, bool warm,
                         LookAhead look, long s0, long count, int shape) {
  // slots [s0, s0 + count) of L.n (count < 0: to the end); s0 a multiple of the shape's block,
  // so the launch's blocks are those of the whole pass
  const long m = count < 0 ? L.n - s0 : std::min(count, L.n - s0);
  if (L.n <= 0 || m <= 0 || shape < 0 || shape >= kForceShapes || s0 % kForceShapeBlock[shape] != 0) return;
  static_assert(kForceShapes == 4 && kForceShapeBlock[0] == 128 && kForceShapeBlock[1] == 96 &&
                    kForceShapeBlock[2] == 64 && kForceShapeBlock[3] == 192, "the instantiated shapes");
  if (shape == 0)
    launch_lists_forces_shape<128, kForceShapeMinb[0]>(L, cur, out, d, flume, nbr, cull, start, order, csort,
                                                       lists, write_ft, uniform, warm, look, s0, m);
  else if (shape == 1)
    launch_lists_forces_shape<96, kForceShapeMinb[1]>(L, cur, out, d, flume, nbr, cull, start, order, csort,
                                                      lists, write_ft, uniform, warm, look, s0, m);
  else if (shape == 2)
    launch_lists_forces_shape<64, kForceShapeMinb[2]>(L, cur, out, d, flume, nbr, cull, start, order, csort,
                                                      lists, write_ft, uniform, warm, look, s0, m);
  else
    launch_lists_forces_shape<192, kForceShapeMinb[3]>(L, cur, out, d, flume, nbr, cull, start, order, csort,
                                                       lists, write_ft, uniform, warm, look, s0, m);
}

void launch_boundary(const Launch &L, Planes cur, DevScalars *d, const int *flume, int routine) {
  if (L.n <= 0) return;
  k_boundary<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, d, flume, routine, L.n);
}

void launch_part(const Launch &L, Planes cur, DevScalars *d, const int *flume, const NbrRec *nbr,
                 const CullRec *cull, const int *start, int sph_id) {
  if (L.n <= 0) return;
  k_part<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, d, flume, nbr, cull, start, sph_id, L.n);
}

void launch_get_accel(const Launch &L, Planes cur, DevScalars *d, const int *flume) {
  if (L.n <= 0) return;
  k_get_accel<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, d, flume, L.n);
}

void launch_finish_verlet(const Launch &L, Planes cur, DevScalars *d, const int *flume) {
  if (L.n <= 0) return;
  k_finish_verlet<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, d, flume, L.n);
}

void launch_clear_forces(const Launch &L, Planes cur) {
  if (L.n <= 0) return;
  k_clear_forces<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, L.n);
}

void launch_advance_time(cudaStream_t st, DevScalars *d) { k_advance_time<<<1, 1, 0, st>>>(d); }

void launch_regrid(const Launch &L, Planes cur, DevScalars *d, const int *flume, int nflumes,
                   long bucket_cap) {
  const unsigned gf = (unsigned)((nflumes + 127) / 128);
  k_bbox_init<<<gf, 128, 0, L.st>>>(d, nflumes);
  if (L.n > 0) k_bbox_reduce<<<grid_for(L.n, 256), 256, 0, L.st>>>(cur, d, flume, L.n);
  k_grid_derive<<<gf, 128, 0, L.st>>>(d, nflumes);
  k_grid_commit<<<1, 1, 0, L.st>>>(d, nflumes, L.n, bucket_cap);
}

void launch_commit_grids(cudaStream_t st, DevScalars *d, int nflumes, long n, long bucket_cap) {
  k_grid_commit<<<1, 1, 0, st>>>(d, nflumes, n, bucket_cap);
}

void launch_aos_to_planes(const Launch &L, const af3d_particle *aos, const double *acc,
                          const double *anga, const int *flume_of_id, Planes cur, long long *id,
                          int *flume, bool keep_order, long s0, long count) {
  const long m = count < 0 ? L.n - s0 : std::min(count, L.n - s0);
  if (L.n <= 0 || m <= 0) return;
  k_aos_to_planes<<<grid_for(m), kBlock, 0, L.st>>>(aos, acc, anga, flume_of_id, cur, id, flume, keep_order, s0,
                                                    L.n);
}

void launch_planes_to_aos(const Launch &L, Planes cur, const long long *id, const int *flume,
                          af3d_particle *aos, double *acc, double *anga, DevScalars *d, long s0, long count) {
  const long m = count < 0 ? L.n - s0 : std::min(count, L.n - s0);
  if (L.n <= 0 || m <= 0) return;
  k_planes_to_aos<<<grid_for(m), kBlock, 0, L.st>>>(cur, id, flume, aos, acc, anga, d, s0, L.n);
}

void launch_contact_pairs(const Launch &L, Planes cur, DevScalars *d, const int *flume,
                          const NbrRec *nbr, const CullRec *cull, const int *start,
                          const long long *id, long long *out, unsigned long long *count, long cap,
                          int active) {
  if (L.n <= 0) return;
  k_contact_pairs<<<grid_for(L.n), kBlock, 0, L.st>>>(cur, d, flume, nbr, cull, start, id, out, count, cap,
                                                      active, L.n);
}

void launch_cells_by_id(const Launch &L, const int *key, const long long *id, DevScalars *d,
                        long long *cell_of_id) {
  if (L.n <= 0) return;
  k_cells_by_id<<<grid_for(L.n), kBlock, 0, L.st>>>(key, id, d, cell_of_id, L.n);
}

#ifdef AF3D_FAST
}  // namespace fast
#endif

}  // namespace af3d
