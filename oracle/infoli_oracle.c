/*
 * InfOli CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-timestep network update,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  The product (libinfoli_gpu.so, infoli.x) never links or
 * calls anything in this file.
 *
 * Parity pin: the FP32 path below is compared byte-for-byte against the
 * untouched reference binaries built by oracle/build_ref.sh (traces in
 * tests/golden/, generated by tests/golden/make_golden.py).
 *
 * Reference anchors (paths inside the reference project):
 *   parameters / default state   bin/default.conf:1-42, src/openmp/infoli.c:240-292
 *   read_parameters              src/utils/utils.c:137-160
 *   read_g_CaL_from_file         src/utils/utils.c:124-135
 *   uniform topology generator   src/openmp/infoli.c:337-375
 *   stimulus schedule            src/openmp/infoli.c:482-485
 *   gap-junction coupling        src/openmp/infoli.c:496-520
 *   fused compartment update     src/openmp/infoli.c:556-679
 *   min()                        src/utils/utils.c:340-343
 *   FP64 twin                    src/single_threaded/infoli.c:371-858 (double, exp, pow)
 *   randomised initial state     src/single_threaded/infoli.c:206-236 (RAND_INIT);
 *                                pinned on that program built with the switch
 *                                at 1 (tests/golden/single_rand_init.npz)
 *
 * Build: gcc -O3 -ffp-contract=off -fopenmp -shared -fPIC (see oracle/Makefile).
 * Contraction is off so the float arithmetic matches the reference build and
 * is the same on x86-64 and aarch64.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Number of per-cell state arrays, in default.conf order (lines 24-42). */
#define ORC_NSTATE 19
enum {
    S_V_DEND = 0, S_CAL_R, S_POT_S, S_HCUR_Q, S_CA2, S_I_CAH, S_G_CAL, S_V_SOMA,
    S_NA_M, S_NA_H, S_POT_N, S_POT_P, S_POT_XS, S_CAL_K, S_CAL_L, S_V_AXON,
    S_NA_MA, S_NA_HA, S_POT_XA
};
/* Model constants, default.conf lines 1-23. */
enum {
    P_DELTA = 0, P_CONDUCTANCE, P_C_M, P_G_NA_S, P_G_KDR_S, P_G_K_S, P_G_LS,
    P_G_K_CA, P_G_CAH, P_G_LD, P_G_H, P_G_NA_A, P_G_NA_R, P_G_K_A, P_G_LA,
    P_P1, P_P2, P_G_INT, P_V_NA, P_V_K, P_V_CA, P_V_H, P_V_L, ORC_NPARAM
};

/* Stimulus kinds: 0 = one global pulse (the reference's hard-coded schedule,
 * src/openmp/infoli.c:482-485: amplitude a for start <= step < end);
 * 1 = per-cell pulse (amp[c] for onset[c] <= step < onset[c] + dur);
 * 2 = per-step table, one row of n values per step from `first` on (the
 * reference's stimulus file, src/utils/utils.c:70-122, applied as in its
 * disabled loop src/openmp/infoli.c:434-477: iAppIn = iAppArray[cell]); 0
 * outside the table. */
typedef struct {
    int kind;
    int start, end;       /* kind 0 */
    float amp;            /* kind 0 */
    const float *cell_amp;  /* kind 1, [n]; kind 2, [rows][n] */
    const int *cell_onset;  /* kind 1, [n] */
    int dur;                /* kind 1; kind 2: rows */
    int n;                  /* kind 2 */
} orc_stim;

static inline float stim_f32(const orc_stim *s, int c, int step) {
    if (s->kind == 0) return (step >= s->start && step < s->end) ? s->amp : 0.0f;
    if (s->kind == 2) {
        const int r = step - s->start;
        return (r >= 0 && r < s->dur) ? s->cell_amp[(size_t)r * s->n + c] : 0.0f;
    }
    return (step >= s->cell_onset[c] && step < s->cell_onset[c] + s->dur) ? s->cell_amp[c] : 0.0f;
}

/* ---------------------------------------------------------------- config --- */

/* read_parameters (src/utils/utils.c:137-160): 42 positional "name = value"
 * lines; names are not checked.  Returns 0, or -(line) of the first bad line,
 * or -1000 if the file cannot be opened. */
int orc_read_parameters(const char *path, float *values) {
    char name[100];
    FILE *fd = fopen(path, "r");
    if (!fd) return -1000;
    for (int i = 0; i < 42; i++) {
        if (fscanf(fd, "%99s = %f\n", name, &values[i]) != 2) {
            fclose(fd);
            return -(i + 1);
        }
    }
    fclose(fd);
    return 0;
}

/* ------------------------------------------------------------- topology --- */

/* The reference's built-in generator (src/openmp/infoli.c:337-375): srand(seed),
 * then for every receiver, for every sender != receiver in ascending order, one
 * rand() draw; the edge exists when (float)rand()/(float)RAND_MAX <= p.
 * Neighbour lists come out in ascending sender id.  Writes CSR row_ptr[n+1]
 * and col[] (capacity cap); returns the edge count, or -1 if cap is too small
 * (row_ptr is still complete in that case). */
long long orc_gen_uniform(int n, float p, unsigned seed, long long *row_ptr, int *col, long long cap) {
    long long e = 0;
    int overflow = 0;
    srand(seed);
    row_ptr[0] = 0;
    for (int r = 0; r < n; r++) {
        for (int s = 0; s < n; s++) {
            if (s == r) continue;
            float rndm = ((float)rand()) / ((float)RAND_MAX);
            if (rndm <= p) {
                if (e < cap) col[e] = s; else overflow = 1;
                e++;
            }
        }
        row_ptr[r + 1] = e;
    }
    return overflow ? -1 : e;
}

/* ------------------------------------------------------ FP32 step (ref) --- */

static inline float min_f32(float a, float b) { return (a < b) ? a : b; }

/* LOOP 1, gap junctions (src/openmp/infoli.c:496-520): serial float sum in
 * neighbour-list order of g * f(V) * V, f(V) = 0.8 exp(-V^2/100) + 0.2. */
static void coupling_f32(int n, const float *vd, const long long *row_ptr, const int *col,
                         const float *g, float g_uniform, float *ic, int nthreads) {
    int c;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (c = 0; c < n; c++) {
        float acc = 0;
        for (long long k = row_ptr[c]; k < row_ptr[c + 1]; k++) {
            float voltage = vd[col[k]];
            float V = vd[c] - voltage;
            float f = 0.8f * expf(-1 * powf(V, 2) / 100) + 0.2f;
            acc += (g ? g[k] : g_uniform) * f * V;
        }
        ic[c] = acc;
    }
}

/* LOOP 2, one cell (src/openmp/infoli.c:556-675).  Gates are advanced first,
 * currents use the new gates, all three voltages use the old voltages; Ca2Plus
 * uses the old I_CaH, alpha_s the old Ca2Plus; x_s and x_a use the literal 0.05. */
static inline void cell_f32(const float *P, float **S, int c, float I_c, float iApp) {
    const float DELTA = P[P_DELTA], C_M = P[P_C_M], G_NA_S = P[P_G_NA_S],
                G_KDR_S = P[P_G_KDR_S], G_K_S = P[P_G_K_S], G_LS = P[P_G_LS],
                G_K_CA = P[P_G_K_CA], G_CAH = P[P_G_CAH], G_LD = P[P_G_LD], G_H = P[P_G_H],
                G_NA_A = P[P_G_NA_A], G_K_A = P[P_G_K_A], G_LA = P[P_G_LA], P1 = P[P_P1],
                P2 = P[P_P2], G_INT = P[P_G_INT], V_NA = P[P_V_NA], V_K = P[P_V_K],
                V_CA = P[P_V_CA], V_H = P[P_V_H], V_L = P[P_V_L];
    float Vd = S[S_V_DEND][c], Vs = S[S_V_SOMA][c], Va = S[S_V_AXON][c];
    float q = S[S_HCUR_Q][c], r = S[S_CAL_R][c], s = S[S_POT_S][c];
    float Ca = S[S_CA2][c], ICaH = S[S_I_CAH][c], gCaL = S[S_G_CAL][c];
    float k = S[S_CAL_K][c], l = S[S_CAL_L][c], h = S[S_NA_H][c];
    float nn = S[S_POT_N][c], pp = S[S_POT_P][c], xs = S[S_POT_XS][c];
    float ha = S[S_NA_HA][c], xa = S[S_POT_XA][c];

    /* dendrite (:560-593) */
    float q_inf = 1 / (1 + expf((Vd + 80) / 4));
    float tau_q = 1 / (expf(-0.086f * Vd - 14.6f) + expf(0.070f * Vd - 1.87f));
    float dq_dt = (q_inf - q) / tau_q;
    q = DELTA * dq_dt + q;
    float alpha_r = 1.7f / (1 + expf(-(Vd - 5) / 13.9f));
    /* removable singularities (0/0 at Vd = -8.5, Vs = -25, Va = -25 in the
     * reference's arithmetic, which then turns the whole network to NaN
     * through the coupling) take their limits; elsewhere the expressions are
     * the reference's */
    float beta_r = (Vd + 8.5f) == 0.0f ? 0.1f : 0.02f * (Vd + 8.5f) / (expf((Vd + 8.5f) / 5) - 1);
    float r_inf = alpha_r / (alpha_r + beta_r);
    float tau_r = 5 / (alpha_r + beta_r);
    float dr_dt = (r_inf - r) / tau_r;
    r = DELTA * dr_dt + r;
    float alpha_s = min_f32((0.00002f * Ca), 0.01f);
    float beta_s = 0.015f;
    float s_inf = alpha_s / (alpha_s + beta_s);
    float tau_s = 1 / (alpha_s + beta_s);
    float ds_dt = (s_inf - s) / tau_s;
    s = DELTA * ds_dt + s;
    float dCa_dt = -3 * ICaH - 0.075f * Ca;
    Ca = DELTA * dCa_dt + Ca;
    float I_sd = (G_INT / (1 - P1)) * (Vd - Vs);
    float I_CaH_temp = G_CAH * powf(r, 2) * (Vd - V_CA);
    float I_K_Ca = G_K_CA * s * (Vd - V_K);
    float I_ld = G_LD * (Vd - V_L);
    float I_h = G_H * q * (Vd - V_H);
    float dVd_dt = (-(I_CaH_temp + I_sd + I_ld + I_K_Ca + I_c + I_h) + iApp) / C_M;
    ICaH = I_CaH_temp;

    /* soma (:598-642) */
    float k_inf = (1 / (1 + expf(-1 * (Vs + 61) / 4.2f)));
    float l_inf = (1 / (1 + expf((Vs + 85.5f) / 8.5f)));
    float tau_k = 1;
    float tau_l = ((20 * expf((Vs + 160) / 30) / (1 + expf((Vs + 84) / 7.3f))) + 35);
    float dk_dt = (k_inf - k) / tau_k;
    float dl_dt = (l_inf - l) / tau_l;
    k = DELTA * dk_dt + k;
    l = DELTA * dl_dt + l;
    float m_inf = 1 / (1 + (expf((-30 - Vs) / 5.5f)));
    float h_inf = 1 / (1 + (expf((-70 - Vs) / -5.8f)));
    float tau_h = 3 * expf((-40 - Vs) / 33);
    float dh_dt = (h_inf - h) / tau_h;
    float m = m_inf;
    h = h + DELTA * dh_dt;
    float n_inf = 1 / (1 + expf((-3 - Vs) / 10));
    float p_inf = 1 / (1 + expf((-51 - Vs) / -12));
    float tau_n = 5 + (47 * expf(-(-50 - Vs) / 900));
    float tau_p = tau_n;
    float dn_dt = (n_inf - nn) / tau_n;
    float dp_dt = (p_inf - pp) / tau_p;
    nn = DELTA * dn_dt + nn;
    pp = DELTA * dp_dt + pp;
    float alpha_x_s = (Vs + 25) == 0.0f ? 1.3f : 0.13f * (Vs + 25) / (1 - expf(-(Vs + 25) / 10));
    float beta_x_s = 1.69f * expf(-0.0125f * (Vs + 35));
    float x_inf_s = alpha_x_s / (alpha_x_s + beta_x_s);
    float tau_x_s = 1 / (alpha_x_s + beta_x_s);
    float dx_dt_s = (x_inf_s - xs) / tau_x_s;
    xs = 0.05f * dx_dt_s + xs;
    float I_ds = (G_INT / P1) * (Vs - Vd);
    float I_CaL = gCaL * powf(k, 3) * l * (Vs - V_CA);
    float I_Na_s = G_NA_S * powf(m, 3) * h * (Vs - V_NA);
    float I_ls = G_LS * (Vs - V_L);
    float I_Kdr_s = G_KDR_S * powf(nn, 4) * (Vs - V_K);
    float I_K_s = G_K_S * powf(xs, 4) * (Vs - V_K);
    float I_as = (G_INT / (1 - P2)) * (Vs - Va);
    float dVs_dt = (-(I_CaL + I_ds + I_as + I_Na_s + I_ls + I_Kdr_s + I_K_s)) / C_M;

    /* axon (:647-668) */
    float m_inf_a = 1 / (1 + (expf((-30 - Va) / 5.5f)));
    float h_inf_a = 1 / (1 + (expf((-60 - Va) / -5.8f)));
    float tau_h_a = 1.5f * expf((-40 - Va) / 33);
    float dh_dt_a = (h_inf_a - ha) / tau_h_a;
    float ma = m_inf_a;
    ha = ha + DELTA * dh_dt_a;
    float alpha_x_a = (Va + 25) == 0.0f ? 1.3f : 0.13f * (Va + 25) / (1 - expf(-(Va + 25) / 10));
    float beta_x_a = 1.69f * expf(-0.0125f * (Va + 35));
    float x_inf_a = alpha_x_a / (alpha_x_a + beta_x_a);
    float tau_x_a = 1 / (alpha_x_a + beta_x_a);
    float dx_dt_a = (x_inf_a - xa) / tau_x_a;
    xa = 0.05f * dx_dt_a + xa;
    float I_Na_a = G_NA_A * powf(ma, 3) * ha * (Va - V_NA);
    float I_la = G_LA * (Va - V_L);
    float I_sa = (G_INT / P2) * (Va - Vs);
    float I_K_a = G_K_A * powf(xa, 4) * (Va - V_K);
    float dVa_dt = (-(I_K_a + I_sa + I_la + I_Na_a)) / C_M;

    /* new voltages (:673-675) */
    S[S_V_DEND][c] = DELTA * dVd_dt + Vd;
    S[S_V_SOMA][c] = DELTA * dVs_dt + Vs;
    S[S_V_AXON][c] = DELTA * dVa_dt + Va;
    S[S_HCUR_Q][c] = q; S[S_CAL_R][c] = r; S[S_POT_S][c] = s;
    S[S_CA2][c] = Ca; S[S_I_CAH][c] = ICaH;
    S[S_CAL_K][c] = k; S[S_CAL_L][c] = l; S[S_NA_M][c] = m; S[S_NA_H][c] = h;
    S[S_POT_N][c] = nn; S[S_POT_P][c] = pp; S[S_POT_XS][c] = xs;
    S[S_NA_MA][c] = ma; S[S_NA_HA][c] = ha; S[S_POT_XA][c] = xa;
}

/*
 * Run nsteps FP32 steps starting at global step index step0.
 *   state     19*n floats, SoA in default.conf order (updated in place)
 *   row_ptr   CSR of senders per receiver (n+1), col senders
 *   g         per-edge conductance, or NULL for g_uniform on every edge
 *   stim_kind 0: stim_i = {start, end}, stim_f = {amp}
 *             1: per-cell cell_amp[n], cell_onset[n], stim_i[0] = duration
 *             2: table cell_amp[rows][n], stim_i = {first step, rows}
 *   trace_every  record after every step s with ((step0+s) % trace_every)==0
 *                (the reference's print rule, src/openmp/infoli.c:682); 0 = off
 *   tr_axon/tr_soma/tr_dend  [ntrace][n] each, any may be NULL
 * Returns the number of trace rows written.
 */
int orc_run_f32(int n, const float *params, float *state,
                const long long *row_ptr, const int *col, const float *g, float g_uniform,
                int stim_kind, const int *stim_i, const float *stim_f,
                const float *cell_amp, const int *cell_onset,
                int step0, int nsteps, int trace_every,
                float *tr_axon, float *tr_soma, float *tr_dend, int nthreads) {
    float *S[ORC_NSTATE];
    for (int i = 0; i < ORC_NSTATE; i++) S[i] = state + (size_t)i * n;
    float *ic = (float *)malloc(sizeof(float) * (n ? n : 1));
    orc_stim st;
    memset(&st, 0, sizeof st);
    st.kind = stim_kind;
    if (stim_kind == 0) { st.start = stim_i[0]; st.end = stim_i[1]; st.amp = stim_f[0]; }
    else if (stim_kind == 2) { st.cell_amp = cell_amp; st.start = stim_i[0]; st.dur = stim_i[1]; st.n = n; }
    else { st.cell_amp = cell_amp; st.cell_onset = cell_onset; st.dur = stim_i[0]; }
    if (nthreads < 1) nthreads = 1;
    int rows = 0;
    for (int t = 0; t < nsteps; t++) {
        int step = step0 + t;
        coupling_f32(n, S[S_V_DEND], row_ptr, col, g, g_uniform, ic, nthreads);
        int c;
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (c = 0; c < n; c++) cell_f32(params, S, c, ic[c], stim_f32(&st, c, step));
        if (trace_every > 0 && (step % trace_every) == 0) {
            size_t o = (size_t)rows * n;
            if (tr_axon) memcpy(tr_axon + o, S[S_V_AXON], sizeof(float) * n);
            if (tr_soma) memcpy(tr_soma + o, S[S_V_SOMA], sizeof(float) * n);
            if (tr_dend) memcpy(tr_dend + o, S[S_V_DEND], sizeof(float) * n);
            rows++;
        }
    }
    free(ic);
    return rows;
}

/* ------------------------------------------------------------- FP64 twin --- */
/* Same update in double with exp/pow and double literals, following the
 * struct form src/single_threaded/infoli.c:371-858 (CompDend, CompSoma,
 * CompAxon, IcNeighbors :544-556).  Parameters come in as doubles. */

static void coupling_f64(int n, const double *vd, const long long *row_ptr, const int *col,
                         const float *g, double g_uniform, double *ic, int nthreads) {
    int c;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (c = 0; c < n; c++) {
        double acc = 0;
        for (long long k = row_ptr[c]; k < row_ptr[c + 1]; k++) {
            double V = vd[c] - vd[col[k]];
            double f = 0.8 * exp(-1 * pow(V, 2) / 100) + 0.2;
            acc += (g ? (double)g[k] : g_uniform) * f * V;
        }
        ic[c] = acc;
    }
}

static inline void cell_f64(const double *P, double **S, int c, double I_c, double iApp) {
    const double DELTA = P[P_DELTA], C_M = P[P_C_M], G_NA_S = P[P_G_NA_S],
                 G_KDR_S = P[P_G_KDR_S], G_K_S = P[P_G_K_S], G_LS = P[P_G_LS],
                 G_K_CA = P[P_G_K_CA], G_CAH = P[P_G_CAH], G_LD = P[P_G_LD], G_H = P[P_G_H],
                 G_NA_A = P[P_G_NA_A], G_K_A = P[P_G_K_A], G_LA = P[P_G_LA], P1 = P[P_P1],
                 P2 = P[P_P2], G_INT = P[P_G_INT], V_NA = P[P_V_NA], V_K = P[P_V_K],
                 V_CA = P[P_V_CA], V_H = P[P_V_H], V_L = P[P_V_L];
    double Vd = S[S_V_DEND][c], Vs = S[S_V_SOMA][c], Va = S[S_V_AXON][c];
    double q = S[S_HCUR_Q][c], r = S[S_CAL_R][c], s = S[S_POT_S][c];
    double Ca = S[S_CA2][c], ICaH = S[S_I_CAH][c], gCaL = S[S_G_CAL][c];
    double k = S[S_CAL_K][c], l = S[S_CAL_L][c], h = S[S_NA_H][c];
    double nn = S[S_POT_N][c], pp = S[S_POT_P][c], xs = S[S_POT_XS][c];
    double ha = S[S_NA_HA][c], xa = S[S_POT_XA][c];

    double q_inf = 1 / (1 + exp((Vd + 80) / 4));
    double tau_q = 1 / (exp(-0.086 * Vd - 14.6) + exp(0.070 * Vd - 1.87));
    q = DELTA * ((q_inf - q) / tau_q) + q;
    double alpha_r = 1.7 / (1 + exp(-(Vd - 5) / 13.9));
    double beta_r = (Vd + 8.5) == 0.0 ? 0.1 : 0.02 * (Vd + 8.5) / (exp((Vd + 8.5) / 5) - 1);
    double r_inf = alpha_r / (alpha_r + beta_r);
    double tau_r = 5 / (alpha_r + beta_r);
    r = DELTA * ((r_inf - r) / tau_r) + r;
    double alpha_s = (0.00002 * Ca < 0.01) ? 0.00002 * Ca : 0.01;
    double beta_s = 0.015;
    double s_inf = alpha_s / (alpha_s + beta_s);
    double tau_s = 1 / (alpha_s + beta_s);
    s = DELTA * ((s_inf - s) / tau_s) + s;
    Ca = DELTA * (-3 * ICaH - 0.075 * Ca) + Ca;
    double I_sd = (G_INT / (1 - P1)) * (Vd - Vs);
    double I_CaH_temp = G_CAH * pow(r, 2) * (Vd - V_CA);
    double I_K_Ca = G_K_CA * s * (Vd - V_K);
    double I_ld = G_LD * (Vd - V_L);
    double I_h = G_H * q * (Vd - V_H);
    double dVd_dt = (-(I_CaH_temp + I_sd + I_ld + I_K_Ca + I_c + I_h) + iApp) / C_M;
    ICaH = I_CaH_temp;

    double k_inf = 1 / (1 + exp(-1 * (Vs + 61) / 4.2));
    double l_inf = 1 / (1 + exp((Vs + 85.5) / 8.5));
    double tau_l = (20 * exp((Vs + 160) / 30) / (1 + exp((Vs + 84) / 7.3))) + 35;
    k = DELTA * (k_inf - k) + k;
    l = DELTA * ((l_inf - l) / tau_l) + l;
    double m = 1 / (1 + exp((-30 - Vs) / 5.5));
    double h_inf = 1 / (1 + exp((-70 - Vs) / -5.8));
    double tau_h = 3 * exp((-40 - Vs) / 33);
    h = h + DELTA * ((h_inf - h) / tau_h);
    double n_inf = 1 / (1 + exp((-3 - Vs) / 10));
    double p_inf = 1 / (1 + exp((-51 - Vs) / -12));
    double tau_n = 5 + (47 * exp(-(-50 - Vs) / 900));
    nn = DELTA * ((n_inf - nn) / tau_n) + nn;
    pp = DELTA * ((p_inf - pp) / tau_n) + pp;
    double alpha_x_s = (Vs + 25) == 0.0 ? 1.3 : 0.13 * (Vs + 25) / (1 - exp(-(Vs + 25) / 10));
    double beta_x_s = 1.69 * exp(-0.0125 * (Vs + 35));
    double x_inf_s = alpha_x_s / (alpha_x_s + beta_x_s);
    double tau_x_s = 1 / (alpha_x_s + beta_x_s);
    xs = 0.05 * ((x_inf_s - xs) / tau_x_s) + xs;
    double I_ds = (G_INT / P1) * (Vs - Vd);
    double I_CaL = gCaL * pow(k, 3) * l * (Vs - V_CA);
    double I_Na_s = G_NA_S * pow(m, 3) * h * (Vs - V_NA);
    double I_ls = G_LS * (Vs - V_L);
    double I_Kdr_s = G_KDR_S * pow(nn, 4) * (Vs - V_K);
    double I_K_s = G_K_S * pow(xs, 4) * (Vs - V_K);
    double I_as = (G_INT / (1 - P2)) * (Vs - Va);
    double dVs_dt = (-(I_CaL + I_ds + I_as + I_Na_s + I_ls + I_Kdr_s + I_K_s)) / C_M;

    double ma = 1 / (1 + exp((-30 - Va) / 5.5));
    double h_inf_a = 1 / (1 + exp((-60 - Va) / -5.8));
    double tau_h_a = 1.5 * exp((-40 - Va) / 33);
    ha = ha + DELTA * ((h_inf_a - ha) / tau_h_a);
    double alpha_x_a = (Va + 25) == 0.0 ? 1.3 : 0.13 * (Va + 25) / (1 - exp(-(Va + 25) / 10));
    double beta_x_a = 1.69 * exp(-0.0125 * (Va + 35));
    double x_inf_a = alpha_x_a / (alpha_x_a + beta_x_a);
    double tau_x_a = 1 / (alpha_x_a + beta_x_a);
    xa = 0.05 * ((x_inf_a - xa) / tau_x_a) + xa;
    double I_Na_a = G_NA_A * pow(ma, 3) * ha * (Va - V_NA);
    double I_la = G_LA * (Va - V_L);
    double I_sa = (G_INT / P2) * (Va - Vs);
    double I_K_a = G_K_A * pow(xa, 4) * (Va - V_K);
    double dVa_dt = (-(I_K_a + I_sa + I_la + I_Na_a)) / C_M;

    S[S_V_DEND][c] = DELTA * dVd_dt + Vd;
    S[S_V_SOMA][c] = DELTA * dVs_dt + Vs;
    S[S_V_AXON][c] = DELTA * dVa_dt + Va;
    S[S_HCUR_Q][c] = q; S[S_CAL_R][c] = r; S[S_POT_S][c] = s;
    S[S_CA2][c] = Ca; S[S_I_CAH][c] = ICaH;
    S[S_CAL_K][c] = k; S[S_CAL_L][c] = l; S[S_NA_M][c] = m; S[S_NA_H][c] = h;
    S[S_POT_N][c] = nn; S[S_POT_P][c] = pp; S[S_POT_XS][c] = xs;
    S[S_NA_MA][c] = ma; S[S_NA_HA][c] = ha; S[S_POT_XA][c] = xa;
}

/* FP64 twin of orc_run_f32: params[23] and state[19*n] are double, traces double. */
int orc_run_f64(int n, const double *params, double *state,
                const long long *row_ptr, const int *col, const float *g, double g_uniform,
                int stim_kind, const int *stim_i, const float *stim_f,
                const float *cell_amp, const int *cell_onset,
                int step0, int nsteps, int trace_every,
                double *tr_axon, double *tr_soma, double *tr_dend, int nthreads) {
    double *S[ORC_NSTATE];
    for (int i = 0; i < ORC_NSTATE; i++) S[i] = state + (size_t)i * n;
    double *ic = (double *)malloc(sizeof(double) * (n ? n : 1));
    if (nthreads < 1) nthreads = 1;
    int rows = 0;
    for (int t = 0; t < nsteps; t++) {
        int step = step0 + t;
        coupling_f64(n, S[S_V_DEND], row_ptr, col, g, g_uniform, ic, nthreads);
        int c;
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (c = 0; c < n; c++) {
            double iapp;
            if (stim_kind == 0) iapp = (step >= stim_i[0] && step < stim_i[1]) ? (double)stim_f[0] : 0.0;
            else if (stim_kind == 2)
                iapp = (step - stim_i[0] >= 0 && step - stim_i[0] < stim_i[1])
                           ? (double)cell_amp[(size_t)(step - stim_i[0]) * n + c] : 0.0;
            else iapp = (step >= cell_onset[c] && step < cell_onset[c] + stim_i[0]) ? (double)cell_amp[c] : 0.0;
            cell_f64(params, S, c, ic[c], iapp);
        }
        if (trace_every > 0 && (step % trace_every) == 0) {
            size_t o = (size_t)rows * n;
            if (tr_axon) memcpy(tr_axon + o, S[S_V_AXON], sizeof(double) * n);
            if (tr_soma) memcpy(tr_soma + o, S[S_V_SOMA], sizeof(double) * n);
            if (tr_dend) memcpy(tr_dend + o, S[S_V_DEND], sizeof(double) * n);
            rows++;
        }
    }
    free(ic);
    return rows;
}

/* Randomised initial state, RAND_INIT (src/single_threaded/infoli.c:206-236;
 * placeholder in src/openmp/infoli.c:402-422): srand(seed); g_CaL[c] = 0.6 +
 * 0.2 * (rand() % 100) / 100 for every cell, then for every cell an odd
 * k = (rand() % ceil(100 / DELTA)) | 1 drawn and the cell run alone (no
 * coupling current, no stimulus).  The reference alternates two state buffers
 * (step j reads buffer j % 2 and writes (j % 2) ^ 1, :227-228) and starts the
 * simulation from buffer 0 (:293, :316), which holds the state after k - 1
 * steps: that state is the result here.  state[19*n] is updated in place; steps_out[n] (may be
 * NULL) receives the drawn k. */
void orc_random_init(int n, const float *params, float *state, unsigned seed, int *steps_out) {
    float *S[ORC_NSTATE];
    for (int i = 0; i < ORC_NSTATE; i++) S[i] = state + (size_t)i * n;
    srand(seed);
    for (int c = 0; c < n; c++) S[S_G_CAL][c] = 0.6 + (0.2 * (rand() % 100) / 100);
    const int span = (int)ceil(100 / params[P_DELTA]);
    for (int c = 0; c < n; c++) {
        const int k = (rand() % span) | 1;
        if (steps_out) steps_out[c] = k;
        for (int j = 0; j < k - 1; j++) cell_f32(params, S, c, 0.0f, 0.0f);
    }
}

/* The same in double (the single-threaded reference's arithmetic: its state
 * and g_CaL draw are doubles, its isolated steps CompDend/CompSoma/CompAxon in
 * double): the FP64 twin's randomised initial state. */
void orc_random_init_f64(int n, const double *params, double *state, unsigned seed, int *steps_out) {
    double *S[ORC_NSTATE];
    for (int i = 0; i < ORC_NSTATE; i++) S[i] = state + (size_t)i * n;
    srand(seed);
    for (int c = 0; c < n; c++) S[S_G_CAL][c] = 0.6 + (0.2 * (rand() % 100) / 100);
    const int span = (int)ceil(100 / params[P_DELTA]);
    for (int c = 0; c < n; c++) {
        const int k = (rand() % span) | 1;
        if (steps_out) steps_out[c] = k;
        for (int j = 0; j < k - 1; j++) cell_f64(params, S, c, 0.0, 0.0);
    }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
