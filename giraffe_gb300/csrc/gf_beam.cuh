// Beam_1 element on the device: Gauss-point kinematics, internal force and
// tangent, and the Gauss-point commit.
//
// Restates reference src/Beam_1.cpp:695-835 (Mount) and 1494-1506
// (SaveLagrange).  One thread owns one element; the internal force and all
// rotation updates are FP64, the tangent is computed in TK (double for the
// plain path, float for the mixed-precision path).  The 9x9 Gauss-point
// operator M = B^T D B + G is rotated to the global frame block by block
// (T3^T M_pq T3) before the DeltaN expansion, which is the same linear map as
// the reference's T^T (DeltaN^T M DeltaN) T on the 18x18 matrix.
#pragma once
#include <type_traits>

#include "gf_math.cuh"
#include "gf_types.h"

namespace gf {

// Interpolated nodal increments at one Gauss point, local frame.
struct BeamInterp {
  V3<double> alpha, dalpha, u, du;
};

// Gauss-point state used by the force and tangent (local frame).
struct BeamGP {
  V3<double> alpha, dalpha, dz;
  double g;
  M3<double> Xi, dXi, Qt;  // Qt = (Q_delta Q_i)^T
  double sig[6];           // retro-rotated stress resultants (n_r, m_r)
};

// reference src/Beam_1.cpp:700-746
GF_HD BeamInterp beam_interp(const BeamConst& c, const double* d, int g) {
  const double* N = c.N[g];
  const double* dN = c.dN[g];
  V3<double> a, da, u, du;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    a[i] = d[3 + i] * N[0] + d[9 + i] * N[1] + d[15 + i] * N[2];
    da[i] = d[3 + i] * dN[0] + d[9 + i] * dN[1] + d[15 + i] * dN[2];
    u[i] = d[i] * N[0] + d[6 + i] * N[1] + d[12 + i] * N[2];
    du[i] = d[i] * dN[0] + d[6 + i] * dN[1] + d[12 + i] * dN[2];
  }
  M3<double> T;
#pragma unroll
  for (int i = 0; i < 9; ++i) T[i] = c.T3[i];
  BeamInterp r;
  r.alpha = mv(T, a);
  r.dalpha = mv(T, da);
  r.u = mv(T, u);
  r.du = mv(T, du);
  return r;
}

// Q_delta and Xi of the incremental rotation (reference src/Beam_1.cpp:748-753)
GF_HD void beam_rot(const V3<double>& alpha, double& g, M3<double>& Qd, M3<double>& Xi) {
  double n2 = dot(alpha, alpha);
  g = 4.0 / (4.0 + n2);
  M3<double> A = skew(alpha), A2 = mul(A, A);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    Qd[i] = g * (A[i] + 0.5 * A2[i]);
    Xi[i] = g * 0.5 * A[i];
  }
  Qd[0] += 1.0; Qd[4] += 1.0; Qd[8] += 1.0;
  Xi[0] += g; Xi[4] += g; Xi[8] += g;
}

// Constitutive product sigma = D eps with D = diag(D00..D55) + D34 (E I12)
GF_HD void beam_stress(const BeamConst& c, const double* eps, double* sig) {
#pragma unroll
  for (int i = 0; i < 6; ++i) sig[i] = c.Dd[i] * eps[i];
  sig[3] += c.D34 * eps[4];
  sig[4] += c.D34 * eps[3];
}

// reference src/Beam_1.cpp:748-788
GF_HD void beam_kinematics(const BeamConst& c, const BeamHist& h, const BeamInterp& ip, int g, BeamGP& k) {
  k.alpha = ip.alpha;
  k.dalpha = ip.dalpha;
  M3<double> Qd;
  beam_rot(ip.alpha, k.g, Qd, k.Xi);
  M3<double> dA = skew(ip.dalpha);
  double ad = dot(ip.alpha, ip.dalpha);
#pragma unroll
  for (int i = 0; i < 9; ++i) k.dXi[i] = -0.5 * k.g * (ad * k.Xi[i] - dA[i]);
  M3<double> Qi;
#pragma unroll
  for (int i = 0; i < 9; ++i) Qi[i] = h.Q[g][i];
#pragma unroll
  for (int i = 0; i < 3; ++i) k.dz[i] = ip.du[i] + h.dz[g][i];
  k.Qt = transpose(mul(Qd, Qi));
  V3<double> eta = mv(k.Qt, k.dz);
  V3<double> t = tmv(k.Xi, ip.dalpha);
  V3<double> kap = tmv(Qi, t);
  double eps[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    eps[i] = eta[i] - c.e3r[i];
    eps[3 + i] = kap[i] + h.kap[g][i];
  }
  beam_stress(c, eps, k.sig);
}

// Gauss-point operator M = B^T D B + G (9x9, local frame, stored at op_idx)
// in TK.
// With B = [[Qt, 0, P], [0, R, S]] (P = Qt dZ Xi, R = Qt Xi, S = Qt dXi) and
// D = diag(Dt, Dr), the blocks are M00 = Qt^T Dt Qt, M02 = Qt^T Dt P,
// M11 = R^T Dr R, M12 = R^T Dr S, M22 = P^T Dt P + S^T Dr S, M20 = M02^T,
// M21 = M12^T, M01 = M10 = 0; G is added on top (reference
// src/Beam_1.cpp:796-822).
template <typename TK> GF_HD M3<TK> xtdy(const M3<TK>& X, const M3<TK>& DY) { return tmul(X, DY); }
template <typename TK> GF_HD M3<TK> diag_rows(const M3<TK>& Y, TK d0, TK d1, TK d2) {
  M3<TK> r;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r[j] = d0 * Y[j];
    r[3 + j] = d1 * Y[3 + j];
    r[6 + j] = d2 * Y[6 + j];
  }
  return r;
}
template <typename TK> GF_HD M3<TK> dr_rows(const M3<TK>& Y, TK d3, TK d4, TK d5, TK d34) {
  M3<TK> r;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    r[j] = d3 * Y[j] + d34 * Y[3 + j];
    r[3 + j] = d34 * Y[j] + d4 * Y[3 + j];
    r[6 + j] = d5 * Y[6 + j];
  }
  return r;
}

// Storage of the 9x9 operator: its 3x3 blocks (0, 1) and (1, 0) are zero
// and are not stored, the other 63 entries row by row: entry (r, c) at
// op_idx(r, c) (rows 0-2 hold columns 0-2 and 6-8, rows 3-5 columns 3-8,
// rows 6-8 all nine).
constexpr int OP_N = 63;
GF_HD constexpr int op_idx(int r, int c) {
  return r < 3 ? r * 6 + (c < 3 ? c : c - 3) : (r < 6 ? 18 + (r - 3) * 6 + (c - 3) : 36 + (r - 6) * 9 + c);
}

template <typename TK>
GF_HD void store_block(TK* M, int ms, int p, int q, const M3<TK>& X, bool add = false, bool transposed = false) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      TK v = transposed ? X[j * 3 + i] : X[i * 3 + j];
      TK& dst = M[op_idx(3 * p + i, 3 * q + j) * ms];
      dst = add ? dst + v : v;
    }
}

template <typename TK>
GF_HD void beam_gp_operator(const BeamConst& c, const BeamGP& k, TK* M, int ms = 1) {
  const double* sig = k.sig;
  M3<double> kdZ = skew(k.dz);
  TK d0 = TK(c.Dd[0]), d1 = TK(c.Dd[1]), d2 = TK(c.Dd[2]);
  TK d3 = TK(c.Dd[3]), d4 = TK(c.Dd[4]), d5 = TK(c.Dd[5]), d34 = TK(c.D34);
  M3<TK> Qt = cvt<TK>(k.Qt);
  M3<TK> Xi = cvt<TK>(k.Xi);
  store_block(M, ms, 0, 0, tmul(Qt, diag_rows(Qt, d0, d1, d2)));
  {
    M3<TK> P = mul(Qt, mul(cvt<TK>(kdZ), Xi));
    M3<TK> DtP = diag_rows(P, d0, d1, d2);
    M3<TK> M02 = tmul(Qt, DtP);
    store_block(M, ms, 0, 2, M02);
    store_block(M, ms, 2, 0, M02, false, true);
    store_block(M, ms, 2, 2, tmul(P, DtP));
  }
  {
    M3<TK> R = mul(Qt, Xi);
    M3<TK> S = mul(Qt, cvt<TK>(k.dXi));
    M3<TK> DrS = dr_rows(S, d3, d4, d5, d34);
    store_block(M, ms, 1, 1, tmul(R, dr_rows(R, d3, d4, d5, d34)));
    M3<TK> M12 = tmul(R, DrS);
    store_block(M, ms, 1, 2, M12);
    store_block(M, ms, 2, 1, M12, false, true);
    store_block(M, ms, 2, 2, tmul(S, DrS), true);
  }
  // G (reference src/Beam_1.cpp:796-822)
  V3<double> nr = {{sig[0], sig[1], sig[2]}}, mr = {{sig[3], sig[4], sig[5]}};
  V3<TK> n = cvt<TK>(tmv(k.Qt, nr)), m = cvt<TK>(tmv(k.Qt, mr));
  V3<TK> al = cvt<TK>(k.alpha);
  TK g = TK(k.g);
  M3<TK> Sn = skew(n);
  {
    M3<TK> Gua = mul(Sn, Xi);
#pragma unroll
    for (int i = 0; i < 9; ++i) Gua[i] = -Gua[i];
    store_block(M, ms, 0, 2, Gua, true);
    store_block(M, ms, 2, 0, tmul(Xi, Sn), true);
  }
  M3<TK> V2 = opV(al, m, g);
  {
    M3<TK> dZ = cvt<TK>(kdZ);
    M3<TK> Gaa = tmul(Xi, mul(mul(dZ, Sn), Xi));
    M3<TK> V1 = opV(al, mv(dZ, n), g);
    M3<TK> dV = opdV(al, cvt<TK>(k.dalpha), m, g);
    M3<TK> SmXi = mul(skew(m), Xi);
    M3<TK> t2 = tmul(cvt<TK>(k.dXi), SmXi);
#pragma unroll
    for (int i = 0; i < 9; ++i) Gaa[i] = Gaa[i] - V1[i] + dV[i] - t2[i];
    store_block(M, ms, 2, 2, Gaa, true);
    M3<TK> t3 = tmul(Xi, SmXi);
#pragma unroll
    for (int i = 0; i < 9; ++i) t3[i] = V2[i] - t3[i];
    store_block(M, ms, 1, 2, t3, true);
  }
  store_block(M, ms, 2, 1, V2, true);
}

// M'_pq = T3^T M_pq T3 for one 3x3 block, in place.
template <typename TK> GF_HD void rotate_block9(const TK* T, TK* M, int ms, int p, int q) {
  TK b[9], t[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) b[i * 3 + j] = M[op_idx(3 * p + i, 3 * q + j) * ms];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) t[i * 3 + j] = b[i * 3] * T[j] + b[i * 3 + 1] * T[3 + j] + b[i * 3 + 2] * T[6 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      M[op_idx(3 * p + i, 3 * q + j) * ms] = T[i] * t[j] + T[3 + i] * t[3 + j] + T[6 + i] * t[6 + j];
}

// M'_pq = T3^T M_pq T3 for the seven 3x3 blocks that are not zero (M01 = M10
// = 0 stay zero), in place.  In FP64 the block loop is unrolled; in FP32-pair
// arithmetic, whose operations are several instructions each, it is kept
// rolled so the kernel's code stays within the instruction cache.
template <typename TK> GF_HD void rotate_blocks9(const BeamConst& c, TK* M, int ms = 1) {
  TK T[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) T[i] = TK(c.T3[i]);
  // blocks (0,0) (0,2) (1,1) (1,2) (2,0) (2,1) (2,2)
  if constexpr (std::is_same<TK, double>::value) {
#pragma unroll
    for (int k = 0; k < 7; ++k)
      rotate_block9(T, M, ms, k < 2 ? 0 : (k < 4 ? 1 : 2), k < 4 ? (k == 0 ? 0 : (k == 2 ? 1 : 2)) : k - 4);
  } else {
#pragma unroll 1
    for (int k = 0; k < 7; ++k)
      rotate_block9(T, M, ms, k < 2 ? 0 : (k < 4 ? 1 : 2), k < 4 ? (k == 0 ? 0 : (k == 2 ? 1 : 2)) : k - 4);
  }
}

// Internal force contribution of one Gauss point, global frame, added to
// f[i * fs] (reference src/Beam_1.cpp:828).
GF_HD void beam_gp_force(const BeamConst& c, const BeamGP& k, int g, double* f, int fs = 1) {
  V3<double> nr = {{k.sig[0], k.sig[1], k.sig[2]}}, mr = {{k.sig[3], k.sig[4], k.sig[5]}};
  V3<double> n = tmv(k.Qt, nr), m = tmv(k.Qt, mr);
  V3<double> s1 = tmv(k.Xi, m);
  V3<double> a1 = tmv(k.Xi, tmv(skew(k.dz), n));
  V3<double> a2 = tmv(k.dXi, m);
  V3<double> s2 = {{a1[0] + a2[0], a1[1] + a2[1], a1[2] + a2[2]}};
  M3<double> T;
#pragma unroll
  for (int i = 0; i < 9; ++i) T[i] = c.T3[i];
  V3<double> g0 = tmv(T, n), g1 = tmv(T, s1), g2 = tmv(T, s2);
  double wJ = c.jac;
#pragma unroll
  for (int I = 0; I < 3; ++I) {
    double dN = c.dN[g][I], N = c.N[g][I];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      f[(6 * I + i) * fs] += wJ * dN * g0[i];
      f[(6 * I + 3 + i) * fs] += wJ * (dN * g1[i] + N * g2[i]);
    }
  }
}

GF_HD double beam_M_entry(const BeamConst& c, const double* D0, const double* D1, int ds, double a1Mr, int r, int s);

// The 6x6 block (I, J) of K_e (global frame) from the two rotated
// Gauss-point operators, written to K (column-major 18x18, leading
// dimension 18, entries ks apart).  The products of the Gauss weight and shape-function values
// and derivatives are formed once per block (cdd = w N'_I N'_J, cdn = w N'_I
// N_J, cnd = w N_I N'_J, cnn = w N_I N_J), so each entry is a short FMA chain
// over the operator blocks: translation rows/columns couple through N' only,
// rotation rows/columns through N' (curvature) and N (the alpha terms).  With
// dyn, the inertial blocks of beam_M_entry are added.
template <typename TK>
GF_HD void beam_K_block(const BeamConst& c, const TK* M0, const TK* M1, int I, int J, int ms, double* K,
                        bool dyn = false, const double* D0 = nullptr, const double* D1 = nullptr, int ds = 1,
                        double a1Mr = 0.0, int64_t ks = 1) {
  TK cdd[2], cdn[2], cnd[2], cnn[2];
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    TK w = TK(c.jac), dNI = TK(c.dN[g][I]), NI = TK(c.N[g][I]), dNJ = TK(c.dN[g][J]), NJ = TK(c.N[g][J]);
    cdd[g] = w * dNI * dNJ;
    cdn[g] = w * dNI * NJ;
    cnd[g] = w * NI * dNJ;
    cnn[g] = w * NI * NJ;
  }
#pragma unroll 1
  for (int b = 0; b < 6; ++b)
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      TK acc = TK(0);
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const TK* M = g ? M1 : M0;
        if (a < 3 && b < 3) {
          acc += cdd[g] * M[op_idx(a, b) * ms];
        } else if (a < 3) {
          // the operator's block (0, 1) is zero
          int bb = b - 3;
          acc += cdn[g] * M[op_idx(a, 6 + bb) * ms];
        } else if (b < 3) {
          // the operator's block (1, 0) is zero
          int aa = a - 3;
          acc += cnd[g] * M[op_idx(6 + aa, b) * ms];
        } else {
          int aa = a - 3, bb = b - 3;
          acc += cdd[g] * M[op_idx(3 + aa, 3 + bb) * ms] + cdn[g] * M[op_idx(3 + aa, 6 + bb) * ms] +
                 cnd[g] * M[op_idx(6 + aa, 3 + bb) * ms] + cnn[g] * M[op_idx(6 + aa, 6 + bb) * ms];
        }
      }
      double k = double(acc);
      if (dyn) k += beam_M_entry(c, D0, D1, ds, a1Mr, 6 * I + a, 6 * J + b);
      K[((6 * I + a) + 18 * (6 * J + b)) * ks] = k;
    }
}

// Inertial contribution of one Gauss point (Beam_1::MountMass, reference
// src/Beam_1.cpp:1564-1638, Hooke sections: no offset of the mass centre).
// In the element frame, with Newmark coefficients a[0..5] = a1..a6:
//   dT_u = Mr (a1 du - a2 v_i - a3 acc_i)
//   dT_a = Xi(da) h,  h = J_i w2 + w1 x J_i w1,  J_i = Q(alpha_i) Jr Q(alpha_i)^T,
//   w1 = a4 da + a5 w_i + a6 dw_i,  w2 = a1 da - a2 w_i - a3 dw_i
// (Newmark in the tangent space transported by Q_delta, and Xi^T Q_delta = Xi
// for Rodrigues parameters), and the exact tangent
//   d dT_u/d du = a1 Mr I,
//   d dT_a/d da = Xi (a1 J_i + a4 (skew(w1) J_i - skew(J_i w1)))
//                 - g^2/2 (h + da x h / 2) da^T - g/2 skew(h).
// Adds wJ N_I dT (global frame) to f[(6I+i)*fs] and returns the rotated
// rotational tangent T3^T (d dT_a/d da) T3 in Daa[q * ds]; the translational
// tangent is a1 Mr I in every frame.
GF_HD void beam_gp_inertia(const BeamConst& c, const BeamHistAux& x, const BeamInterp& ip, const double* vel,
                           const double* acc, const double* a, int g, double* f, int fs, double* Daa, int ds) {
  const double* N = c.N[g];
  M3<double> T;
#pragma unroll
  for (int i = 0; i < 9; ++i) T[i] = c.T3[i];
  V3<double> wi, dwi, vi, ai;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    wi[i] = vel[3 + i] * N[0] + vel[9 + i] * N[1] + vel[15 + i] * N[2];
    dwi[i] = acc[3 + i] * N[0] + acc[9 + i] * N[1] + acc[15 + i] * N[2];
    vi[i] = vel[i] * N[0] + vel[6 + i] * N[1] + vel[12 + i] * N[2];
    ai[i] = acc[i] * N[0] + acc[6 + i] * N[1] + acc[12 + i] * N[2];
  }
  wi = mv(T, wi);
  dwi = mv(T, dwi);
  vi = mv(T, vi);
  ai = mv(T, ai);
  const double a1 = a[0], a2 = a[1], a3 = a[2], a4 = a[3], a5 = a[4], a6 = a[5];
  V3<double> fu;
#pragma unroll
  for (int i = 0; i < 3; ++i) fu[i] = c.Mr * (a1 * ip.u[i] - a2 * vi[i] - a3 * ai[i]);
  V3<double> al = {{x.alpha[g][0], x.alpha[g][1], x.alpha[g][2]}};
  M3<double> Qi = rodrigues(al), Jr;
#pragma unroll
  for (int i = 0; i < 9; ++i) Jr[i] = c.Jr[i];
  M3<double> Ji = mul(mul(Qi, Jr), transpose(Qi));
  V3<double> w1, w2;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    w1[i] = a4 * ip.alpha[i] + a5 * wi[i] + a6 * dwi[i];
    w2[i] = a1 * ip.alpha[i] - a2 * wi[i] - a3 * dwi[i];
  }
  V3<double> Jw1 = mv(Ji, w1), Jw2 = mv(Ji, w2), cr = cross(w1, Jw1), h;
#pragma unroll
  for (int i = 0; i < 3; ++i) h[i] = Jw2[i] + cr[i];
  double gg;
  M3<double> Qd, Xi;
  beam_rot(ip.alpha, gg, Qd, Xi);
  V3<double> m = mv(Xi, h);
  M3<double> t = mul(skew(w1), Ji), SJw1 = skew(Jw1), Dh;
#pragma unroll
  for (int q = 0; q < 9; ++q) Dh[q] = a1 * Ji[q] + a4 * (t[q] - SJw1[q]);
  M3<double> D = mul(Xi, Dh);
  V3<double> axh = cross(ip.alpha, h);
  M3<double> Sh = skew(h);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      D[i * 3 + j] += -0.5 * gg * gg * (h[i] + 0.5 * axh[i]) * ip.alpha[j] - 0.5 * gg * Sh[i * 3 + j];
  M3<double> Dg = tmul(T, mul(D, T));
#pragma unroll
  for (int q = 0; q < 9; ++q) Daa[q * ds] = Dg[q];
  V3<double> gu = tmv(T, fu), ga = tmv(T, m);
  double wJ = c.jac;
#pragma unroll
  for (int I = 0; I < 3; ++I)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      f[(6 * I + i) * fs] += wJ * N[I] * gu[i];
      f[(6 * I + 3 + i) * fs] += wJ * N[I] * ga[i];
    }
}

// Inertial tangent entry (row r, column s of the 18x18, global frame).
GF_HD double beam_M_entry(const BeamConst& c, const double* D0, const double* D1, int ds, double a1Mr, int r, int s) {
  int I = r / 6, a = r % 6, J = s / 6, b = s % 6;
  double acc = 0.0;
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    double w = c.jac * c.N[g][I] * c.N[g][J];
    if (a < 3 && b < 3) {
      if (a == b) acc += w * a1Mr;
    } else if (a >= 3 && b >= 3) {
      const double* D = g ? D1 : D0;
      acc += w * D[((a - 3) * 3 + (b - 3)) * ds];
    }
  }
  return acc;
}

// reference src/Beam_1.cpp:1494-1506
GF_HD void beam_commit(const BeamConst& c, BeamHist& h, BeamHistAux& x, const double* d) {
#pragma unroll 1
  for (int g = 0; g < 2; ++g) {
    BeamInterp ip = beam_interp(c, d, g);
    BeamGP k;
    beam_kinematics(c, h, ip, g, k);
    double gg;
    M3<double> Qd, Xi;
    beam_rot(ip.alpha, gg, Qd, Xi);
    M3<double> Qi;
#pragma unroll
    for (int i = 0; i < 9; ++i) Qi[i] = h.Q[g][i];
    M3<double> Q = mul(Qd, Qi);
    // kappa_r (reference src/Beam_1.cpp:785) recomputed for the history
    V3<double> t = tmv(Xi, ip.dalpha);
    V3<double> kap = tmv(Qi, t);
#pragma unroll
    for (int i = 0; i < 9; ++i) h.Q[g][i] = Q[i];
    V3<double> ai = {{x.alpha[g][0], x.alpha[g][1], x.alpha[g][2]}};
    V3<double> an = rodrigues_compose(ip.alpha, ai);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      x.u[g][i] += ip.u[i];
      h.kap[g][i] = kap[i] + h.kap[g][i];
      h.dz[g][i] = k.dz[i];
      x.alpha[g][i] = an[i];
    }
  }
}

}  // namespace gf
