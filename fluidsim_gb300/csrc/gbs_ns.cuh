// Device helpers shared by the generic and the compile-time-size ns kernels:
// RK4 stage selector and arguments, dissipation frequency, the per-mode RK4
// update, the fused projection / dealiasing / stage epilogue, and the block
// max reduction used for the CFL condition.
#pragma once

#include "gbs_core.cuh"

namespace gbs {

// Stage selector for the last pass of a tendency evaluation: the plain
// tendency, the four RK4 stages, forward Euler, the two RK2 stages and the
// two RK2_trapezoid (Heun) stages of TimeSteppingPseudoSpectral.  Final
// stages write the new state (projected, dealiased, NaN-checked).
enum Mode {
  kTend = 0, kRK0 = 1, kRK1 = 2, kRK2 = 3, kRK3 = 4,
  kEuler = 5, kR2a = 6, kR2b = 7, kHeunA = 8, kHeunB = 9,
  // phase-shift schemes (the shifted evaluations divide their tendency by
  // the phase factor before the stage formula)
  kStoreTmp = 10,   // tmp  = N
  kStoreTmp1 = 11,  // tmp1 = N
  kStoreTmp2 = 12,  // tmp2 = N
  kEulerPS = 13,    // S <- (S + dt (tmp + N~)/2) E
  kPS2a = 14,       // tmp = (S + dt N) E, tmp1 = N
  kPS2b = 15,       // S <- S E + dt E2 (tmp1 + N~)/2
  kPSXb = 16,       // tmp1 = Nd0 = (tmp1 + N~)/2, tmp = (S + dt Nd0) E
  kPSXd = 17        // S <- S E + dt E2 (tmp1 + (tmp2 + N~)/2)/2
};

__device__ __forceinline__ bool final_stage(int mode) {
  return mode == kRK3 || mode == kEuler || mode == kR2b || mode == kHeunB ||
         mode == kEulerPS || mode == kPS2b || mode == kPSXd;
}

// Phase factor exp(i phi), phi = sx kx + sy ky + sz kz, of the phase-shift
// schemes: shift lengths (dx, dy, dz) / 2 for the fixed shift
// (pseudo_spect.py:282-300), alpha_i d_i or beta_i d_i for the random ones
// (operators3d.py:1128-1146, operators2d.py:618-631); computed in the
// working precision from the wavenumbers of the mode.
// sin and cos of pi x: the argument reduction of sincospi is exact and
// short (no large-argument path, which would cost local memory in every
// kernel that carries the phase-shift branch)
__device__ __forceinline__ void tsincospi(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ void tsincospi(double x, double* s, double* c) { sincospi(x, s, c); }

template <typename C, typename T>
__device__ __forceinline__ C phase_factor(T sx, T sy, T sz, T kx, T ky, T kz) {
  const T phi = sx * kx + sy * ky + sz * kz;
  T sn, cs;
  tsincospi(phi * T(0.31830988618379067154), &sn, &cs);  // phi / pi
  return mk<C>(cs, sn);
}

struct RKArgs {
  const void* S;  // state (read) for the stages that use S_0
  void* Sout;     // state (write) for the final stages
  void* tmp;      // _state_spect_tmp
  void* tmp1;     // _state_spect_tmp1
  void* tend;     // output for kTend
  double dt;
  float fdt;  // dt rounded to float (the FP32 kernels read this one)
  int* nan_flag;
  const void* add;  // optional forcing (nvar spectral fields) added to the
                    // tendency before projection and dealiasing
  void* tmp2;       // third buffer of RK2_phaseshift_exact
  int phase;        // divide the tendency by exp(i phi) (shifted evaluation)
  double sx, sy, sz;  // phase shift lengths (phi = sx kx + sy ky + sz kz)
  const void* in;   // state the tendency is evaluated on (ns3d.strat: b, vz)
};

// Viscosities for sigma(k) = f_d + f_d_hypo.
struct Phys {
  double nu2, nu4, nu8, num4;
  double k2_hypo0;  // K2 at (0, .., 1): the value f_d_hypo[0, .., 0] copies
  float fnu2, fnu4, fnu8, fnum4, fk2_hypo0;  // the same rounded to float
  int proj;         // ns3d projection: GBS_PROJ_PERPK / _TOROIDAL / _POLOIDAL
  int no_vz_kz0;    // ns3d: vz(kz = 0) = 0 after the projection
};

// FP32 kernels read float copies of the double parameters made on the host
// (or once per thread), so that no FP64 instruction runs per mode: GB300
// executes FP64 at 2 operations per clock per SM against 128 for FP32.
template <typename T>
__device__ __forceinline__ T dt_of(const RKArgs& a) {
  if constexpr (sizeof(T) == 8) return a.dt;
  else return a.fdt;
}

// fluidsim/base/solvers/pseudo_spect.py:166-191
template <typename T>
__device__ __forceinline__ T freq_lin(const Phys& q, T k2, bool k0) {
  if constexpr (sizeof(T) == 4) {  // the same operations on the float copies
    float fd = q.fnu2 > 0.f ? q.fnu2 * k2 : 0.f;
    if (q.fnu4 > 0.f) fd += q.fnu4 * (k2 * k2);
    if (q.fnu8 > 0.f) {
      const float k4 = k2 * k2;
      fd += q.fnu8 * (k4 * k4);
    }
    if (q.fnum4 != 0.f) {
      const float k2n0 = k0 ? q.fk2_hypo0 : k2;
      fd += q.fnum4 / (k2n0 * k2n0);
    }
    return fd;
  }
  T fd = q.nu2 > 0 ? T(q.nu2) * k2 : T(0);
  if (q.nu4 > 0) fd += T(q.nu4) * (k2 * k2);
  if (q.nu8 > 0) {
    T k4 = k2 * k2;
    fd += T(q.nu8) * (k4 * k4);
  }
  if (q.num4 != 0) {
    T k2n0 = k0 ? T(q.k2_hypo0) : k2;
    fd += T(q.num4) / (k2n0 * k2n0);
  }
  return fd;
}

__device__ __forceinline__ double dexp(double x) { return exp(x); }
__device__ __forceinline__ float dexp(float x) { return expf(x); }

// New state of a final stage at one mode, before projection and
// dealiasing (same evaluation order as the numpy expressions):
//   kRK3   tmp + dt/6 N3                         pseudo_spect.py:984
//   kEuler (S + dt N) E                          pseudo_spect.py:51-60,279
//   kR2b   S E + dt E2 N                         pseudo_spect.py:63-67,517
//   kHeunB tmp1 + dt/2 N, tmp1 = (S + dt/2 N0) E pseudo_spect.py:567-569
// EXT: compiled with the modes of the schemes other than RK4 (the fast
// kernels instantiate an RK4-only variant, which keeps their epilogue lean).
template <typename C, typename T, bool EXT>
__device__ __forceinline__ C final_value(int mode, const RKArgs& a, int64_t i, C N, T sigma) {
  const T dt = dt_of<T>(a);
  if (!EXT || mode == kRK3) {
    const C t = static_cast<const C*>(a.tmp)[i];
    const T c6 = dt / T(6);
    return mk<C>(t.x + c6 * N.x, t.y + c6 * N.y);
  }
  if (mode == kHeunB) {
    const C t = static_cast<const C*>(a.tmp1)[i];
    const T c2 = dt / T(2);
    return mk<C>(t.x + c2 * N.x, t.y + c2 * N.y);
  }
  const C S = static_cast<const C*>(a.S)[i];
  const T E = dexp(-dt * sigma);
  if (mode == kEuler) return cscale(mk<C>(S.x + dt * N.x, S.y + dt * N.y), E);
  if (mode == kEulerPS) {  // pseudo_spect.py:409-419
    const C t = static_cast<const C*>(a.tmp)[i];
    const C Nd = cscale(cadd(t, N), T(0.5));
    return cscale(mk<C>(S.x + dt * Nd.x, S.y + dt * Nd.y), E);
  }
  C Nd = N;  // kR2b
  if (mode == kPS2b) {  // pseudo_spect.py:624-639
    Nd = cscale(cadd(static_cast<const C*>(a.tmp1)[i], N), T(0.5));
  } else if (mode == kPSXd) {  // pseudo_spect.py:784-796
    const C n1 = cscale(cadd(static_cast<const C*>(a.tmp2)[i], N), T(0.5));
    Nd = cscale(cadd(static_cast<const C*>(a.tmp1)[i], n1), T(0.5));
  }
  const T E2 = dexp(-dt / T(2) * sigma);
  const T c1 = dt * E2;
  return mk<C>(S.x * E + c1 * Nd.x, S.y * E + c1 * Nd.y);
}

// RK4 stages 0-2 on values: S = S_0, t = tmp (read at stages 1 and 2);
// pseudo_spect.py:898-984, same evaluation order as the numpy expressions.
template <typename C, typename T>
__device__ __forceinline__ void rk4_stage_values(int mode, T dt, T sigma, C N, C S, C t,
                                                 C& tmp_out, C& tmp1_out) {
  if (mode == kRK0) {
    T E = dexp(-dt * sigma), E2 = dexp(-dt / T(2) * sigma);
    T c6 = dt / T(6), c2 = dt / T(2);
    tmp_out = cscale(mk<C>(S.x + c6 * N.x, S.y + c6 * N.y), E);
    tmp1_out = cscale(mk<C>(S.x + c2 * N.x, S.y + c2 * N.y), E2);
  } else if (mode == kRK1) {
    T E2 = dexp(-dt / T(2) * sigma);
    T c3 = dt / T(3) * E2, c2 = dt / T(2);
    tmp_out = mk<C>(t.x + c3 * N.x, t.y + c3 * N.y);
    tmp1_out = mk<C>(S.x * E2 + c2 * N.x, S.y * E2 + c2 * N.y);
  } else {  // kRK2
    T E = dexp(-dt * sigma), E2 = dexp(-dt / T(2) * sigma);
    T c3 = dt / T(3) * E2, c1 = dt * E2;
    tmp_out = mk<C>(t.x + c3 * N.x, t.y + c3 * N.y);
    tmp1_out = mk<C>(S.x * E + c1 * N.x, S.y * E + c1 * N.y);
  }
}

// Intermediate stage update at one mode (RK4: pseudo_spect.py:898-984;
// RK2 first stage: 505-512; RK2_trapezoid first stage: 559-567), same
// evaluation order as the numpy expressions there.
template <typename C, typename T, bool EXT>
__device__ __forceinline__ void rk_update(int mode, const RKArgs& a, int64_t i,
                                         C N, T sigma) {
  const T dt = dt_of<T>(a);
  C* tmp = static_cast<C*>(a.tmp);
  C* tmp1 = static_cast<C*>(a.tmp1);
  if (!EXT && mode > kRK2) return;
  if (mode >= kRK0 && mode <= kRK2) {
    const C S = static_cast<const C*>(a.S)[i];
    const C t = mode == kRK0 ? mk<C>(0, 0) : tmp[i];
    C o, o1;
    rk4_stage_values<C, T>(mode, dt, sigma, N, S, t, o, o1);
    tmp[i] = o;
    tmp1[i] = o1;
  } else if (!EXT) {
    return;
  } else if (mode == kR2a) {
    const C S = static_cast<const C*>(a.S)[i];
    const T E2 = dexp(-dt / T(2) * sigma);
    const T c2 = dt / T(2);
    tmp[i] = cscale(mk<C>(S.x + c2 * N.x, S.y + c2 * N.y), E2);
  } else if (mode == kHeunA) {
    const C S = static_cast<const C*>(a.S)[i];
    const T E = dexp(-dt * sigma);
    const T c2 = dt / T(2);
    tmp[i] = cscale(mk<C>(S.x + dt * N.x, S.y + dt * N.y), E);
    tmp1[i] = cscale(mk<C>(S.x + c2 * N.x, S.y + c2 * N.y), E);
  } else if (mode == kStoreTmp) {
    tmp[i] = N;
  } else if (mode == kStoreTmp1) {
    tmp1[i] = N;
  } else if (mode == kStoreTmp2) {
    static_cast<C*>(a.tmp2)[i] = N;
  } else if (mode == kPS2a) {  // pseudo_spect.py:617-620
    const C S = static_cast<const C*>(a.S)[i];
    const T E = dexp(-dt * sigma);
    tmp[i] = cscale(mk<C>(S.x + dt * N.x, S.y + dt * N.y), E);
    tmp1[i] = N;
  } else if (mode == kPSXb) {  // pseudo_spect.py:759-767
    const C S = static_cast<const C*>(a.S)[i];
    const T E = dexp(-dt * sigma);
    const C Nd0 = cscale(cadd(tmp1[i], N), T(0.5));
    tmp1[i] = Nd0;
    tmp[i] = cscale(mk<C>(S.x + dt * Nd0.x, S.y + dt * Nd0.y), E);
  }
}

// N / exp(i phi) for the shifted evaluations (|exp(i phi)| = 1: times the
// conjugate)
template <typename C, typename T>
__device__ __forceinline__ C unshift(const RKArgs& a, C N, T kx, T ky, T kz) {
  const C e = phase_factor<C, T>(T(a.sx), T(a.sy), T(a.sz), kx, ky, kz);
  return cmulc(N, e);
}

// project_perpk3d: v -= k (k.v)/|k|^2; the k = 0 mode is left unchanged
template <typename C, typename T, int NV>
__device__ __forceinline__ void project3(C (&v)[NV], T kx, T ky, T kz, T k2, bool k0) {
  if (k0) return;
  const T inv = crcp(k2);
  C t = mk<C>((kx * v[0].x + ky * v[1].x + kz * v[2].x) * inv,
              (kx * v[0].y + ky * v[1].y + kz * v[2].y) * inv);
  v[0] = csub(v[0], cscale(t, kx));
  v[1] = csub(v[1], cscale(t, ky));
  v[2] = csub(v[2], cscale(t, kz));
}

// toroidal projection, operators3d.py:911-959: v = (e_phi . v) e_phi
template <typename C, typename T, int NV>
__device__ __forceinline__ void project_toroidal(C (&v)[NV], T kx, T ky) {
  T kh2 = kx * kx + ky * ky;
  if (kh2 == T(0)) kh2 = T(1e-14);
  const T t = sqrt(T(1) / kh2);
  const T cp = kx * t, sp = ky * t;
  const C tmp = cadd(cscale(v[0], -sp), cscale(v[1], cp));
  v[0] = cscale(tmp, -sp);
  v[1] = cscale(tmp, cp);
  v[2] = mk<C>(0, 0);
}

// poloidal projection, operators3d.py:788-855: v = (e_theta . v) e_theta
template <typename C, typename T, int NV>
__device__ __forceinline__ void project_poloidal(C (&v)[NV], T kx, T ky, T kz) {
  const T kh2 = kx * kx + ky * ky;
  T k2n = kh2 + kz * kz, kh2n = kh2;
  if (kh2n == T(0)) kh2n = T(1e-14);
  if (k2n == T(0)) k2n = T(1e-14);
  const T inv_kh2 = T(1) / kh2n, inv_k2 = T(1) / k2n;
  const T ct = kz * sqrt(inv_k2), st = sqrt(kh2 * inv_k2);
  const T cp = kx * sqrt(inv_kh2), sp = ky * sqrt(inv_kh2);
  const T a = ct * cp, b = ct * sp;
  const C tmp = csub(cadd(cscale(v[0], a), cscale(v[1], b)), cscale(v[2], st));
  v[0] = cscale(tmp, a);
  v[1] = cscale(tmp, b);
  v[2] = cscale(tmp, -st);
}

// project_state_spect, ns3d/solver.py:255-263: the velocity (v[0..2]) is
// projected; no_vz_kz0 zeroes vz and, with a buoyancy field (nv = 4), b at
// kz = 0
template <typename C, typename T, int NV, bool EXT = true>
__device__ __forceinline__ void project_state(const Phys& q, C (&v)[NV], T kx, T ky,
                                              T kz, T k2, bool k0) {
  if (!EXT) {  // the default projector only
    project3(v, kx, ky, kz, k2, k0);
    return;
  }
  if (q.proj == 1) project_toroidal(v, kx, ky);
  else if (q.proj == 2) project_poloidal(v, kx, ky, kz);
  else project3(v, kx, ky, kz, k2, k0);
  if (q.no_vz_kz0 && kz == T(0)) {
    v[2] = mk<C>(0, 0);
    if (NV == 4) v[NV - 1] = mk<C>(0, 0);
  }
}

// ns3d epilogue at one mode for NV state fields (3: ns3d; 4: ns3d.strat,
// velocity then buoyancy): N (already scaled by 1/N) -> projection,
// dealiasing, then the stage `mode` (ns3d/solver.py:251-252,
// ns3d/strat/solver.py:209-216, ns3d/time_stepping.py:12-20).
// EXT: compiled with the modes of the other schemes, the phase-shift branch
// and the other projections (the fast kernels instantiate a variant for RK4
// with the default projector).
// The lean epilogue (RK4 stages, plain tendency, default projector) of one
// position whose S_0 and tmp values the caller loaded (S0, T0; as many as
// the stage reads): a pass can then load several positions' values before
// storing any.  Same operations as stage_epilogue3<..., false>.
template <typename C, typename T, int NV>
__device__ __forceinline__ void stage_epilogue_rk4(int mode, const RKArgs& a, int64_t i,
                                                   int64_t nK, C (&N)[NV], const C (&S0)[NV],
                                                   const C (&T0)[NV], T kx, T ky, T kz, T k2,
                                                   bool k0, bool rm, const Phys& q) {
  project3(N, kx, ky, kz, k2, k0);
  if (rm) N[0] = N[1] = N[2] = N[NV - 1] = mk<C>(0, 0);
  if (mode == kTend) {
    C* o = static_cast<C*>(a.tend);
#pragma unroll
    for (int f = 0; f < NV; ++f) o[i + f * nK] = N[f];
  } else if (mode == kRK3) {
    const T c6 = dt_of<T>(a) / T(6);
    C Sn[NV];
#pragma unroll
    for (int f = 0; f < NV; ++f) Sn[f] = mk<C>(T0[f].x + c6 * N[f].x, T0[f].y + c6 * N[f].y);
    project3(Sn, kx, ky, kz, k2, k0);
    if (rm) Sn[0] = Sn[1] = Sn[2] = Sn[NV - 1] = mk<C>(0, 0);
    C* So = static_cast<C*>(a.Sout);
#pragma unroll
    for (int f = 0; f < NV; ++f) So[i + f * nK] = Sn[f];
    if (isnan(Sn[0].x) || isnan(Sn[0].y)) atomicOr(a.nan_flag, 1);
  } else {
    const T sig = freq_lin<T>(q, k2, k0);
    C* tmp = static_cast<C*>(a.tmp);
    C* tmp1 = static_cast<C*>(a.tmp1);
#pragma unroll
    for (int f = 0; f < NV; ++f) {
      C o, o1;
      rk4_stage_values<C, T>(mode, dt_of<T>(a), sig, N[f], S0[f], T0[f], o, o1);
      tmp[i + f * nK] = o;
      tmp1[i + f * nK] = o1;
    }
  }
}

template <typename C, typename T, int NV, bool EXT = true>
__device__ __forceinline__ void stage_epilogue3(int mode, const RKArgs& a, int64_t i,
                                                int64_t nK, C (&N)[NV], T kx, T ky,
                                                T kz, T k2, bool k0, bool rm,
                                                const Phys& q) {
  if constexpr (!EXT) {  // RK4 stages and plain tendencies, default projector
    // (zeroing by explicit assignments: the same as unrolled loops, but
    // ptxas allocates the unrolled-loop form with spills here)
    project3(N, kx, ky, kz, k2, k0);
    if (rm) N[0] = N[1] = N[2] = N[NV - 1] = mk<C>(0, 0);
    if (mode == kTend) {
      C* o = static_cast<C*>(a.tend);
#pragma unroll
      for (int f = 0; f < NV; ++f) o[i + f * nK] = N[f];
    } else if (mode == kRK3) {
      const C* tmp = static_cast<const C*>(a.tmp);
      const T c6 = dt_of<T>(a) / T(6);
      C Sn[NV];
#pragma unroll
      for (int f = 0; f < NV; ++f) {
        const C t = tmp[i + f * nK];
        Sn[f] = mk<C>(t.x + c6 * N[f].x, t.y + c6 * N[f].y);
      }
      project3(Sn, kx, ky, kz, k2, k0);
      if (rm) Sn[0] = Sn[1] = Sn[2] = Sn[NV - 1] = mk<C>(0, 0);
      C* So = static_cast<C*>(a.Sout);
#pragma unroll
      for (int f = 0; f < NV; ++f) So[i + f * nK] = Sn[f];
      if (isnan(Sn[0].x) || isnan(Sn[0].y)) atomicOr(a.nan_flag, 1);
    } else {
      const T sig = freq_lin<T>(q, k2, k0);
#pragma unroll
      for (int f = 0; f < NV; ++f) rk_update<C, T, false>(mode, a, i + f * nK, N[f], sig);
    }
    return;
  }
  project_state<C, T, NV, EXT>(q, N, kx, ky, kz, k2, k0);
  if (rm) N[0] = N[1] = N[2] = N[NV - 1] = mk<C>(0, 0);
  if (EXT && a.phase) {
    const C e = phase_factor<C, T>(T(a.sx), T(a.sy), T(a.sz), kx, ky, kz);
#pragma unroll
    for (int f = 0; f < NV; ++f) N[f] = cmulc(N[f], e);
  }
  if (mode == kTend) {
    C* o = static_cast<C*>(a.tend);
#pragma unroll
    for (int f = 0; f < NV; ++f) o[i + f * nK] = N[f];
  } else if (EXT ? final_stage(mode) : mode == kRK3) {
    const T sig = (mode == kRK3 || mode == kHeunB) ? T(0) : freq_lin<T>(q, k2, k0);
    C Sn[NV];
#pragma unroll
    for (int f = 0; f < NV; ++f) Sn[f] = final_value<C, T, EXT>(mode, a, i + f * nK, N[f], sig);
    project_state<C, T, NV, EXT>(q, Sn, kx, ky, kz, k2, k0);
    if (rm) Sn[0] = Sn[1] = Sn[2] = Sn[NV - 1] = mk<C>(0, 0);
    C* So = static_cast<C*>(a.Sout);
#pragma unroll
    for (int f = 0; f < NV; ++f) So[i + f * nK] = Sn[f];
    if (isnan(Sn[0].x) || isnan(Sn[0].y)) atomicOr(a.nan_flag, 1);
  } else {
    const T sig = freq_lin<T>(q, k2, k0);
#pragma unroll
    for (int f = 0; f < NV; ++f) rk_update<C, T, EXT>(mode, a, i + f * nK, N[f], sig);
  }
}

// ns2d epilogue at one mode (no projection).
template <typename C, typename T, bool EXT = true>
__device__ __forceinline__ void stage_epilogue1(int mode, const RKArgs& a, int64_t i,
                                                C N, T kx, T ky, bool k0, bool rm,
                                                const Phys& q) {
  const T k2 = kx * kx + ky * ky;
  if (rm) N = mk<C>(0, 0);
  if (EXT && a.phase) N = unshift<C, T>(a, N, kx, ky, T(0));
  if (mode == kTend) {
    static_cast<C*>(a.tend)[i] = N;
  } else if (EXT ? final_stage(mode) : mode == kRK3) {
    const T sig = (mode == kRK3 || mode == kHeunB) ? T(0) : freq_lin<T>(q, k2, k0);
    C Sn = final_value<C, T, EXT>(mode, a, i, N, sig);
    if (rm) Sn = mk<C>(0, 0);
    static_cast<C*>(a.Sout)[i] = Sn;
    if (isnan(Sn.x) || isnan(Sn.y)) atomicOr(a.nan_flag, 1);
  } else {
    rk_update<C, T, EXT>(mode, a, i, N, freq_lin<T>(q, k2, k0));
  }
}

// Block-wide max of three non-negative values, folded into dst[0..2] (the
// bit patterns of non-negative doubles order like the values).  Every
// thread of the block must call it.
template <typename T>
__device__ __forceinline__ void block_max3(T a, T b, T c, unsigned long long* dst) {
  __shared__ double red[3][32];
  double v[3] = {(double)a, (double)b, (double)c};
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o; o >>= 1) v[k] = fmax(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    if (lane == 0) red[k][w] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double x = lane < nw ? red[k][lane] : 0.0;
      for (int o = 16; o; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
      if (lane == 0) atomicMax(dst + k, (unsigned long long)__double_as_longlong(x));
    }
  }
}

}  // namespace gbs
