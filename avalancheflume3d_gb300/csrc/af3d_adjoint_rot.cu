// af3d_adjoint_rot.cu -- reverse of the predictor (init_Verlet) and of the start-up pass.
//
// These kernels recompute only the rotation update of the step they reverse, to form its
// derivative: no branch depends on a recomputed value, so they are compiled with contracted
// multiply-adds (-fmad=true), unlike the contact re-evaluation in af3d_adjoint.cu.
#include "af3d_adjoint.cuh"

namespace af3d {

namespace {

// Reverse of init_Verlet for one clump: from the adjoints of r1, v1, w1, R1 and the sphere
// centres (in + acc + rb) to the adjoint of this step's state (out; out.a/out.al already hold
// the finish terms).  tape: this step's state before the predictor.
__global__ void __launch_bounds__(kAdjBlock) k_adj_predict(Planes P, Planes tape, Planes in, Planes out, Planes acc,
                                                           Planes rb, DevScalars *d, const int *__restrict__ flume,
                                                           long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const DevFlume &fl = d->flumes[flume[s]];
  const double dt = fl.sys.dt, hdt = fl.sys.hdt;
  const V3 r = ld3(tape, AR, s), w = ld3(tape, AW, s), al = ld3(tape, AAL, s);
  if (is_removed(d->time_prev, r.x, fl.sys.side.x)) {
    for (int k = 0; k < NADJ; k++) out.p[k][s] = 0.0;
    return;
  }
  double R[3][3];
  for (int i = 0; i < 3; i++) {
    const V3 row = ld3(tape, ARM + 3 * i, s);
    R[i][0] = row.x; R[i][1] = row.y; R[i][2] = row.z;
  }
  V3 r1_b = ld3(in, AR, s) + ld3(acc, CR, s);
  const V3 v1_b = ld3(acc, CV, s), w1_b = ld3(acc, CW, s);
  V3 Rb3[3] = {ld3(rb, 0, s), ld3(rb, 3, s), ld3(rb, 6, s)};
  fold_spheres(acc, s, P.p[RAD][s] / kROOT2, r1_b, Rb3);
  double R1b[3][3];
  for (int i = 0; i < 3; i++) {
    R1b[i][0] = Rb3[i].x; R1b[i][1] = Rb3[i].y; R1b[i][2] = Rb3[i].z;
  }
  // forward re-evaluation of the rotation update
  const V3 dO = mk(dt * (w.x + hdt * al.x), dt * (w.y + hdt * al.y), dt * (w.z + hdt * al.z));
  const double mag = sqrt(dO.x * dO.x + dO.y * dO.y + dO.z * dO.z);
  double dR[3][3];
  V3 u = mk(0.0, 0.0, 0.0);
  double c = 1.0, sn = 0.0, omc = 0.0;
  const double imag = mag > 0.0 ? 1.0 / mag : 0.0;
  if (mag > 0.0) {
    u = mk(dO.x * imag, dO.y * imag, dO.z * imag);
    if (mag < 0.03125) {
      // Maclaurin series of sin(t)/t and (1 - cos t)/t^2 (first omitted terms below 2^-53 of
      // the sums for t < 2^-5): the derivative needs no bit-exact sine or cosine
      const double t2 = mag * mag;
      const double A = 1.0 - t2 * (1.0 / 6.0) * (1.0 - t2 * (1.0 / 20.0) * (1.0 - t2 * (1.0 / 42.0) *
                                                                              (1.0 - t2 * (1.0 / 72.0))));
      const double Bq = 0.5 * (1.0 - t2 * (1.0 / 12.0) * (1.0 - t2 * (1.0 / 30.0) * (1.0 - t2 * (1.0 / 56.0) *
                                                                                      (1.0 - t2 * (1.0 / 90.0)))));
      sn = A * mag;
      omc = t2 * Bq;
      c = 1.0 - omc;
    } else {
      c = cos(mag);
      sn = sin(mag);
      omc = 1.0 - c;
    }
    const double uu[3] = {u.x, u.y, u.z};
    const double ux[3][3] = {{0.0, -u.z, u.y}, {u.z, 0.0, -u.x}, {-u.y, u.x, 0.0}};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) dR[i][j] = omc * uu[i] * uu[j] + (i == j ? c : 0.0) + sn * ux[i][j];
  } else {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) dR[i][j] = i == j ? 1.0 : 0.0;
  }
  double T[3][3], nrm[3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) T[i][j] = dR[i][0] * R[0][j] + dR[i][1] * R[1][j] + dR[i][2] * R[2][j];
  for (int j = 0; j < 3; j++) nrm[j] = sqrt(T[0][j] * T[0][j] + T[1][j] * T[1][j] + T[2][j] * T[2][j]);
  // column normalisation R1_ij = T_ij / n_j (the derivative needs no bit-exact quotient: one
  // reciprocal per column)
  double Tb[3][3];
  for (int j = 0; j < 3; j++) {
    const double in = 1.0 / nrm[j];
    double q[3], sj = 0.0;
    for (int i = 0; i < 3; i++) {
      q[i] = T[i][j] * in;
      sj += R1b[i][j] * q[i];
    }
    for (int i = 0; i < 3; i++) Tb[i][j] = (R1b[i][j] - q[i] * sj) * in;
  }
  // T = dR R
  double G[3][3], Rb0[3][3];
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) {
      G[i][k] = Tb[i][0] * R[k][0] + Tb[i][1] * R[k][1] + Tb[i][2] * R[k][2];
      Rb0[i][k] = dR[0][i] * Tb[0][k] + dR[1][i] * Tb[1][k] + dR[2][i] * Tb[2][k];
    }
  // dR = c I + sn [u]x + (1 - c) u u^T,  u = dO / |dO|,  c = cos |dO|,  sn = sin |dO|
  const V3 skew = mk(G[2][1] - G[1][2], G[0][2] - G[2][0], G[1][0] - G[0][1]);
  V3 dO_b;
  if (mag > 0.0) {
    const double uu[3] = {u.x, u.y, u.z};
    double c_b = G[0][0] + G[1][1] + G[2][2], ub[3];
    for (int i = 0; i < 3; i++) {
      double a2 = 0.0;
      for (int j = 0; j < 3; j++) {
        c_b -= G[i][j] * uu[i] * uu[j];
        a2 += (G[i][j] + G[j][i]) * uu[j];
      }
      ub[i] = omc * a2;
    }
    const double sn_b = dot(u, skew);
    ub[0] += sn * skew.x;
    ub[1] += sn * skew.y;
    ub[2] += sn * skew.z;
    const double mag_b = -sn * c_b + c * sn_b;
    const V3 u_b = mk(ub[0], ub[1], ub[2]);
    dO_b = imag * (u_b - dot(u, u_b) * u) + mag_b * u;
  } else {
    dO_b = skew;   // dR = I + [dO]x to first order
  }
  // r1 = r + dt (v + hdt a);  v1 = v + dt a;  w1 = w + dt al;  dO = dt (w + hdt al)
  st3(out, AR, s, r1_b);
  st3(out, AV, s, dt * r1_b + v1_b);
  st3(out, AA, s, ld3(out, AA, s) + (dt * hdt) * r1_b + dt * v1_b);
  st3(out, AW, s, w1_b + dt * dO_b);
  st3(out, AAL, s, ld3(out, AAL, s) + dt * w1_b + (dt * hdt) * dO_b);
  for (int i = 0; i < 3; i++) st3(out, ARM + 3 * i, s, mk(Rb0[i][0], Rb0[i][1], Rb0[i][2]));
}

// The start-up force pass (no predictor): the adjoint of the initial state is in + the pass's
// contributions (acc, rb, sphere centres).
__global__ void k_adj_startup(Planes P, Planes in, Planes out, Planes acc, Planes rb, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  V3 r_b = ld3(in, AR, s) + ld3(acc, CR, s);
  V3 Rb3[3] = {ld3(rb, 0, s), ld3(rb, 3, s), ld3(rb, 6, s)};
  fold_spheres(acc, s, P.p[RAD][s] / kROOT2, r_b, Rb3);
  st3(out, AR, s, r_b);
  st3(out, AV, s, ld3(in, AV, s) + ld3(acc, CV, s));
  st3(out, AW, s, ld3(in, AW, s) + ld3(acc, CW, s));
  for (int i = 0; i < 3; i++) st3(out, ARM + 3 * i, s, Rb3[i]);
  st3(out, AA, s, mk(0.0, 0.0, 0.0));
  st3(out, AAL, s, mk(0.0, 0.0, 0.0));
}

}  // namespace

void launch_adj_predict(const Launch &L, Planes P, Planes tape, Planes in, Planes out, Planes acc, Planes rb,
                        DevScalars *d, const int *flume) {
  if (L.n <= 0) return;
  k_adj_predict<<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, tape, in, out, acc, rb, d, flume, L.n);
}

void launch_adj_startup(const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb) {
  if (L.n <= 0) return;
  k_adj_startup<<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, in, out, acc, rb, L.n);
}

}  // namespace af3d
