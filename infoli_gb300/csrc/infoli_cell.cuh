// InfOli 3-compartment cell update on the GPU.  Follows the reference's
// fused compartment loop (src/openmp/infoli.c:556-675; struct form
// CompDend/CompSoma/CompAxon in src/single_threaded/infoli.c:371-858)
// operation for operation:
//   * gates are advanced first, currents use the new gates, every voltage
//     derivative uses the old voltages;
//   * Ca2Plus is advanced from the old I_CaH, alpha_s uses the old Ca2Plus;
//   * x_s and x_a are advanced with the literal 0.05 (not DELTA);
//   * Sodium_m / Sodium_m_a are instantaneous (m = m_inf).
// GPU choices: accurate expf and IEEE division as in the reference; powf with
// an integer exponent is written as products; the Ca2+ concentration is kept
// and advanced in FP64 (the only FP64 arithmetic on the GPU).
//
// The update is cut into eight independent gate units (each advances its
// gates and returns the ionic current(s) they drive) plus one voltage step
// that adds the currents in the reference's order.  The units only read the
// old voltages, so they can run on different warps, and before the
// gap-junction current of the step is known.
#pragma once
#include <cuda_runtime.h>

namespace infoli {

// Model constants, in bin/default.conf order (lines 1-23).
struct ModelParams {
  float DELTA, CONDUCTANCE, C_M, G_NA_S, G_KDR_S, G_K_S, G_LS, G_K_CA, G_CAH, G_LD, G_H,
      G_NA_A, G_NA_R, G_K_A, G_LA, P1, P2, G_INT, V_NA, V_K, V_CA, V_H, V_L;
};

struct Volts {
  float Vd, Vs, Va;  // dendrite / soma / axon
};

// Gate state of one cell (plus g_CaL, constant per cell).
struct Gates {
  float q, r, s;               // Hcurrent_q, Calcium_r, Potassium_s
  double Ca;                   // Ca2Plus (FP64)
  float ICaH;                  // I_CaH (previous step's high-threshold Ca current)
  float gCaL;                  // g_CaL
  float k, l, m, h, n, p, xs;  // Calcium_k/l, Sodium_m/h, Potassium_n/p/x_s
  float ma, ha, xa;            // Sodium_m_a, Sodium_h_a, Potassium_x_a
};

// Ionic currents produced by the gate units.
struct Currents {
  float I_h, I_CaH, I_K_Ca;               // dendrite
  float I_CaL, I_Na_s, I_Kdr_s, I_K_s;    // soma
  float I_Na_a, I_K_a;                    // axon
};

enum { kUnits = 8 };

__device__ __forceinline__ float sq(float x) { return x * x; }

// ---- dendrite (src/openmp/infoli.c:560-593)
// unit 0: H current gate q
__device__ __forceinline__ void unit_q(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vd = v.Vd;
  const float q_inf = 1.0f / (1.0f + expf((Vd + 80.0f) / 4.0f));
  const float tau_q = 1.0f / (expf(-0.086f * Vd - 14.6f) + expf(0.070f * Vd - 1.87f));
  g.q = P.DELTA * ((q_inf - g.q) / tau_q) + g.q;
  c.I_h = P.G_H * g.q * (Vd - P.V_H);
}
// unit 1: high-threshold Ca gate r, Ca-dependent K gate s, Ca2+ concentration
__device__ __forceinline__ void unit_rs(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vd = v.Vd;
  const float alpha_r = 1.7f / (1.0f + expf(-(Vd - 5.0f) / 13.9f));
  // removable singularity at Vd = -8.5 (0/0 in the reference's arithmetic):
  // the limit 0.02 * 5 is used there
  const float xr = Vd + 8.5f;
  const float beta_r = xr == 0.0f ? 0.1f : 0.02f * xr / (expf(xr / 5.0f) - 1.0f);
  const float r_inf = alpha_r / (alpha_r + beta_r);
  const float tau_r = 5.0f / (alpha_r + beta_r);
  g.r = P.DELTA * ((r_inf - g.r) / tau_r) + g.r;
  const float alpha_s = fminf(0.00002f * (float)g.Ca, 0.01f);
  const float beta_s = 0.015f;
  const float s_inf = alpha_s / (alpha_s + beta_s);
  const float tau_s = 1.0f / (alpha_s + beta_s);
  g.s = P.DELTA * ((s_inf - g.s) / tau_s) + g.s;
  {  // FP64 Ca2+ concentration from the old I_CaH and old Ca2Plus (:583-584)
    const double dCa_dt = -3.0 * (double)g.ICaH - 0.075 * g.Ca;
    g.Ca = (double)P.DELTA * dCa_dt + g.Ca;
  }
  c.I_CaH = P.G_CAH * sq(g.r) * (Vd - P.V_CA);
  c.I_K_Ca = P.G_K_CA * g.s * (Vd - P.V_K);
  g.ICaH = c.I_CaH;
}

// ---- soma (:598-642)
// unit 2: low-threshold Ca gates k, l
__device__ __forceinline__ void unit_kl(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vs = v.Vs;
  const float k_inf = 1.0f / (1.0f + expf(-(Vs + 61.0f) / 4.2f));
  const float l_inf = 1.0f / (1.0f + expf((Vs + 85.5f) / 8.5f));
  const float tau_l = (20.0f * expf((Vs + 160.0f) / 30.0f) / (1.0f + expf((Vs + 84.0f) / 7.3f))) + 35.0f;
  g.k = P.DELTA * (k_inf - g.k) + g.k;  // tau_k = 1
  g.l = P.DELTA * ((l_inf - g.l) / tau_l) + g.l;
  c.I_CaL = g.gCaL * (g.k * g.k * g.k) * g.l * (Vs - P.V_CA);
}
// unit 3: Na gates m (instantaneous), h
__device__ __forceinline__ void unit_mh(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vs = v.Vs;
  const float m_inf = 1.0f / (1.0f + expf((-30.0f - Vs) / 5.5f));
  const float h_inf = 1.0f / (1.0f + expf((-70.0f - Vs) / -5.8f));
  const float tau_h = 3.0f * expf((-40.0f - Vs) / 33.0f);
  g.m = m_inf;
  g.h = g.h + P.DELTA * ((h_inf - g.h) / tau_h);
  c.I_Na_s = P.G_NA_S * (g.m * g.m * g.m) * g.h * (Vs - P.V_NA);
}
// unit 4: delayed-rectifier K gates n, p (p is advanced but drives no current)
__device__ __forceinline__ void unit_np(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vs = v.Vs;
  const float n_inf = 1.0f / (1.0f + expf((-3.0f - Vs) / 10.0f));
  const float p_inf = 1.0f / (1.0f + expf((-51.0f - Vs) / -12.0f));
  const float tau_n = 5.0f + (47.0f * expf(-(-50.0f - Vs) / 900.0f));
  g.n = P.DELTA * ((n_inf - g.n) / tau_n) + g.n;
  g.p = P.DELTA * ((p_inf - g.p) / tau_n) + g.p;
  c.I_Kdr_s = P.G_KDR_S * sq(sq(g.n)) * (Vs - P.V_K);
}
// unit 5: voltage-dependent K gate x_s (literal 0.05 step, :632)
__device__ __forceinline__ void unit_xs(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Vs = v.Vs;
  // removable singularity at Vs = -25: the limit 0.13 * 10 is used there
  const float xs = Vs + 25.0f;
  const float alpha_x_s = xs == 0.0f ? 1.3f : 0.13f * xs / (1.0f - expf(-xs / 10.0f));
  const float beta_x_s = 1.69f * expf(-0.0125f * (Vs + 35.0f));
  const float x_inf_s = alpha_x_s / (alpha_x_s + beta_x_s);
  const float tau_x_s = 1.0f / (alpha_x_s + beta_x_s);
  g.xs = 0.05f * ((x_inf_s - g.xs) / tau_x_s) + g.xs;
  c.I_K_s = P.G_K_S * sq(sq(g.xs)) * (Vs - P.V_K);
}

// ---- axon (:647-668)
// unit 6: Na gates m_a (instantaneous), h_a
__device__ __forceinline__ void unit_mha(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Va = v.Va;
  const float m_inf_a = 1.0f / (1.0f + expf((-30.0f - Va) / 5.5f));
  const float h_inf_a = 1.0f / (1.0f + expf((-60.0f - Va) / -5.8f));
  const float tau_h_a = 1.5f * expf((-40.0f - Va) / 33.0f);
  g.ma = m_inf_a;
  g.ha = g.ha + P.DELTA * ((h_inf_a - g.ha) / tau_h_a);
  c.I_Na_a = P.G_NA_A * (g.ma * g.ma * g.ma) * g.ha * (Va - P.V_NA);
}
// unit 7: K gate x_a (literal 0.05 step, :661)
__device__ __forceinline__ void unit_xa(const ModelParams& P, const Volts& v, Gates& g, Currents& c) {
  const float Va = v.Va;
  // removable singularity at Va = -25: the limit 0.13 * 10 is used there
  const float xa = Va + 25.0f;
  const float alpha_x_a = xa == 0.0f ? 1.3f : 0.13f * xa / (1.0f - expf(-xa / 10.0f));
  const float beta_x_a = 1.69f * expf(-0.0125f * (Va + 35.0f));
  const float x_inf_a = alpha_x_a / (alpha_x_a + beta_x_a);
  const float tau_x_a = 1.0f / (alpha_x_a + beta_x_a);
  g.xa = 0.05f * ((x_inf_a - g.xa) / tau_x_a) + g.xa;
  c.I_K_a = P.G_K_A * sq(sq(g.xa)) * (Va - P.V_K);
}

// Run the units whose bit is set in `mask` (bit u = unit u).
__device__ __forceinline__ void run_units(const ModelParams& P, unsigned mask, const Volts& v, Gates& g,
                                          Currents& c) {
  if (mask & 0x01u) unit_q(P, v, g, c);
  if (mask & 0x02u) unit_rs(P, v, g, c);
  if (mask & 0x04u) unit_kl(P, v, g, c);
  if (mask & 0x08u) unit_mh(P, v, g, c);
  if (mask & 0x10u) unit_np(P, v, g, c);
  if (mask & 0x20u) unit_xs(P, v, g, c);
  if (mask & 0x40u) unit_mha(P, v, g, c);
  if (mask & 0x80u) unit_xa(P, v, g, c);
}

// Inter-compartment coupling coefficients of the voltage step.  The reference
// evaluates G_INT / (1 - P1) etc. per cell and step; they depend on the
// parameters only, so they are evaluated once (same IEEE float operations,
// hence the same values).  Division by C_M is skipped when C_M == 1 (x / 1 is
// exactly x), the default.
struct VoltCoef {
  float k_sd, k_ds, k_as, k_sa;
  bool cm_one;
};

__device__ __forceinline__ VoltCoef volt_coef(const ModelParams& P) {
  VoltCoef k;
  k.k_sd = P.G_INT / (1.0f - P.P1);
  k.k_ds = P.G_INT / P.P1;
  k.k_as = P.G_INT / (1.0f - P.P2);
  k.k_sa = P.G_INT / P.P2;
  k.cm_one = P.C_M == 1.0f;
  return k;
}

// Voltage step (:587-592, :635-642, :664-675): currents summed in the
// reference's order, all from the old voltages.  I_c: gap-junction current.
__device__ __forceinline__ void voltage_step(const ModelParams& P, const VoltCoef& k, Volts& v, const Currents& c,
                                             float I_c, float iApp) {
  const float Vd = v.Vd, Vs = v.Vs, Va = v.Va;
  const float I_sd = k.k_sd * (Vd - Vs);
  const float I_ld = P.G_LD * (Vd - P.V_L);
  float dVd_dt = -(c.I_CaH + I_sd + I_ld + c.I_K_Ca + I_c + c.I_h) + iApp;
  const float I_ds = k.k_ds * (Vs - Vd);
  const float I_ls = P.G_LS * (Vs - P.V_L);
  const float I_as = k.k_as * (Vs - Va);
  float dVs_dt = -(c.I_CaL + I_ds + I_as + c.I_Na_s + I_ls + c.I_Kdr_s + c.I_K_s);
  const float I_la = P.G_LA * (Va - P.V_L);
  const float I_sa = k.k_sa * (Va - Vs);
  float dVa_dt = -(c.I_K_a + I_sa + I_la + c.I_Na_a);
  if (!k.cm_one) {
    dVd_dt = dVd_dt / P.C_M;
    dVs_dt = dVs_dt / P.C_M;
    dVa_dt = dVa_dt / P.C_M;
  }
  v.Vd = P.DELTA * dVd_dt + Vd;
  v.Vs = P.DELTA * dVs_dt + Vs;
  v.Va = P.DELTA * dVa_dt + Va;
}

// The whole step of one cell on one thread.
__device__ __forceinline__ void cell_step(const ModelParams& P, Volts& v, Gates& g, float I_c, float iApp) {
  Currents c;
  run_units(P, 0xffu, v, g, c);
  voltage_step(P, volt_coef(P), v, c, I_c, iApp);
}

}  // namespace infoli
