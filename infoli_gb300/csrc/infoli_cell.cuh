// InfOli 3-compartment cell update on the GPU: one thread per cell, state in
// registers.  Follows the reference's fused compartment loop
// (src/openmp/infoli.c:556-675; struct form CompDend/CompSoma/CompAxon in
// src/single_threaded/infoli.c:371-858) operation for operation:
//   * gates are advanced first, currents use the new gates, every voltage
//     derivative uses the old voltages;
//   * Ca2Plus is advanced from the old I_CaH, alpha_s uses the old Ca2Plus;
//   * x_s and x_a are advanced with the literal 0.05 (not DELTA);
//   * Sodium_m / Sodium_m_a are instantaneous (m = m_inf).
// GPU choices: accurate expf and IEEE division as in the reference; powf with
// an integer exponent is written as products; the Ca2+ concentration is kept
// and advanced in FP64 (the only FP64 arithmetic on the GPU).
#pragma once
#include <cuda_runtime.h>

namespace infoli {

// Model constants, in bin/default.conf order (lines 1-23).
struct ModelParams {
  float DELTA, CONDUCTANCE, C_M, G_NA_S, G_KDR_S, G_K_S, G_LS, G_K_CA, G_CAH, G_LD, G_H,
      G_NA_A, G_NA_R, G_K_A, G_LA, P1, P2, G_INT, V_NA, V_K, V_CA, V_H, V_L;
};

// Evolving per-cell state (plus g_CaL, which is constant per cell).
struct CellState {
  float Vd, Vs, Va;       // dendrite / soma / axon voltages
  float q, r, s;          // Hcurrent_q, Calcium_r, Potassium_s
  double Ca;              // Ca2Plus (FP64)
  float ICaH;             // I_CaH
  float gCaL;             // g_CaL
  float k, l, m, h, n, p, xs;  // Calcium_k/l, Sodium_m/h, Potassium_n/p/x_s
  float ma, ha, xa;       // Sodium_m_a, Sodium_h_a, Potassium_x_a
};

__device__ __forceinline__ float sq(float x) { return x * x; }

// One explicit-Euler step of one cell.  I_c: gap-junction current into the
// dendrite; iApp: applied dendritic current.
__device__ __forceinline__ void cell_step(const ModelParams& P, CellState& c, float I_c, float iApp) {
  const float Vd = c.Vd, Vs = c.Vs, Va = c.Va;

  // ---- dendrite (src/openmp/infoli.c:560-593)
  const float q_inf = 1.0f / (1.0f + expf((Vd + 80.0f) / 4.0f));
  const float tau_q = 1.0f / (expf(-0.086f * Vd - 14.6f) + expf(0.070f * Vd - 1.87f));
  c.q = P.DELTA * ((q_inf - c.q) / tau_q) + c.q;
  const float alpha_r = 1.7f / (1.0f + expf(-(Vd - 5.0f) / 13.9f));
  const float beta_r = 0.02f * (Vd + 8.5f) / (expf((Vd + 8.5f) / 5.0f) - 1.0f);
  const float r_inf = alpha_r / (alpha_r + beta_r);
  const float tau_r = 5.0f / (alpha_r + beta_r);
  c.r = P.DELTA * ((r_inf - c.r) / tau_r) + c.r;
  const float ca_f = (float)c.Ca;
  const float alpha_s = fminf(0.00002f * ca_f, 0.01f);
  const float beta_s = 0.015f;
  const float s_inf = alpha_s / (alpha_s + beta_s);
  const float tau_s = 1.0f / (alpha_s + beta_s);
  c.s = P.DELTA * ((s_inf - c.s) / tau_s) + c.s;
  {  // FP64 Ca2+ concentration, old I_CaH and old Ca2Plus (:583-584)
    const double dCa_dt = -3.0 * (double)c.ICaH - 0.075 * c.Ca;
    c.Ca = (double)P.DELTA * dCa_dt + c.Ca;
  }
  const float I_sd = (P.G_INT / (1.0f - P.P1)) * (Vd - Vs);
  const float I_CaH = P.G_CAH * sq(c.r) * (Vd - P.V_CA);
  const float I_K_Ca = P.G_K_CA * c.s * (Vd - P.V_K);
  const float I_ld = P.G_LD * (Vd - P.V_L);
  const float I_h = P.G_H * c.q * (Vd - P.V_H);
  const float dVd_dt = (-(I_CaH + I_sd + I_ld + I_K_Ca + I_c + I_h) + iApp) / P.C_M;
  c.ICaH = I_CaH;

  // ---- soma (:598-642)
  const float k_inf = 1.0f / (1.0f + expf(-(Vs + 61.0f) / 4.2f));
  const float l_inf = 1.0f / (1.0f + expf((Vs + 85.5f) / 8.5f));
  const float tau_l = (20.0f * expf((Vs + 160.0f) / 30.0f) / (1.0f + expf((Vs + 84.0f) / 7.3f))) + 35.0f;
  c.k = P.DELTA * (k_inf - c.k) + c.k;  // tau_k = 1
  c.l = P.DELTA * ((l_inf - c.l) / tau_l) + c.l;
  const float m_inf = 1.0f / (1.0f + expf((-30.0f - Vs) / 5.5f));
  const float h_inf = 1.0f / (1.0f + expf((-70.0f - Vs) / -5.8f));
  const float tau_h = 3.0f * expf((-40.0f - Vs) / 33.0f);
  c.m = m_inf;
  c.h = c.h + P.DELTA * ((h_inf - c.h) / tau_h);
  const float n_inf = 1.0f / (1.0f + expf((-3.0f - Vs) / 10.0f));
  const float p_inf = 1.0f / (1.0f + expf((-51.0f - Vs) / -12.0f));
  const float tau_n = 5.0f + (47.0f * expf(-(-50.0f - Vs) / 900.0f));
  c.n = P.DELTA * ((n_inf - c.n) / tau_n) + c.n;
  c.p = P.DELTA * ((p_inf - c.p) / tau_n) + c.p;
  const float alpha_x_s = 0.13f * (Vs + 25.0f) / (1.0f - expf(-(Vs + 25.0f) / 10.0f));
  const float beta_x_s = 1.69f * expf(-0.0125f * (Vs + 35.0f));
  const float x_inf_s = alpha_x_s / (alpha_x_s + beta_x_s);
  const float tau_x_s = 1.0f / (alpha_x_s + beta_x_s);
  c.xs = 0.05f * ((x_inf_s - c.xs) / tau_x_s) + c.xs;
  const float I_ds = (P.G_INT / P.P1) * (Vs - Vd);
  const float I_CaL = c.gCaL * (c.k * c.k * c.k) * c.l * (Vs - P.V_CA);
  const float I_Na_s = P.G_NA_S * (c.m * c.m * c.m) * c.h * (Vs - P.V_NA);
  const float I_ls = P.G_LS * (Vs - P.V_L);
  const float I_Kdr_s = P.G_KDR_S * sq(sq(c.n)) * (Vs - P.V_K);
  const float I_K_s = P.G_K_S * sq(sq(c.xs)) * (Vs - P.V_K);
  const float I_as = (P.G_INT / (1.0f - P.P2)) * (Vs - Va);
  const float dVs_dt = (-(I_CaL + I_ds + I_as + I_Na_s + I_ls + I_Kdr_s + I_K_s)) / P.C_M;

  // ---- axon (:647-668)
  const float m_inf_a = 1.0f / (1.0f + expf((-30.0f - Va) / 5.5f));
  const float h_inf_a = 1.0f / (1.0f + expf((-60.0f - Va) / -5.8f));
  const float tau_h_a = 1.5f * expf((-40.0f - Va) / 33.0f);
  c.ma = m_inf_a;
  c.ha = c.ha + P.DELTA * ((h_inf_a - c.ha) / tau_h_a);
  const float alpha_x_a = 0.13f * (Va + 25.0f) / (1.0f - expf(-(Va + 25.0f) / 10.0f));
  const float beta_x_a = 1.69f * expf(-0.0125f * (Va + 35.0f));
  const float x_inf_a = alpha_x_a / (alpha_x_a + beta_x_a);
  const float tau_x_a = 1.0f / (alpha_x_a + beta_x_a);
  c.xa = 0.05f * ((x_inf_a - c.xa) / tau_x_a) + c.xa;
  const float I_Na_a = P.G_NA_A * (c.ma * c.ma * c.ma) * c.ha * (Va - P.V_NA);
  const float I_la = P.G_LA * (Va - P.V_L);
  const float I_sa = (P.G_INT / P.P2) * (Va - Vs);
  const float I_K_a = P.G_K_A * sq(sq(c.xa)) * (Va - P.V_K);
  const float dVa_dt = (-(I_K_a + I_sa + I_la + I_Na_a)) / P.C_M;

  // ---- new voltages (:673-675)
  c.Vd = P.DELTA * dVd_dt + Vd;
  c.Vs = P.DELTA * dVs_dt + Vs;
  c.Va = P.DELTA * dVa_dt + Va;
}

}  // namespace infoli
