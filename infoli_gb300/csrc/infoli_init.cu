// Randomised initial states: every cell runs a random number of steps on its
// own (no coupling current, no stimulus) from the configured state, as the
// reference's RAND_INIT does (src/single_threaded/infoli.c:206-236; a
// placeholder in src/openmp/infoli.c:402-422).  The draws use the C library's
// rand() in the reference's order; the isolated steps run on the GPU, one
// thread per cell.  The reference draws an odd count k and alternates its two
// state buffers, step j writing buffer (j % 2) ^ 1 (:227-228), so the last
// step lands in buffer 1 while the simulation starts from buffer 0 (:293,
// :316): the state it starts from is the one after k - 1 steps, and that is
// what is computed here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/infoli_gpu.h"
#include "infoli_cell.cuh"
#include "infoli_internal.h"

namespace infoli {
namespace {

// st: the 19 state arrays of n cells (reference order, INFOLI_S_*).
__global__ void isolated_steps_kernel(const ModelParams P, float* __restrict__ st, int n,
                                      const int* __restrict__ steps) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const size_t N = (size_t)n;
  Volts v;
  Gates g;
  v.Vd = st[0 * N + c];
  g.r = st[1 * N + c];
  g.s = st[2 * N + c];
  g.q = st[3 * N + c];
  g.Ca = (double)st[4 * N + c];
  g.ICaH = st[5 * N + c];
  g.gCaL = st[6 * N + c];
  v.Vs = st[7 * N + c];
  g.m = st[8 * N + c];
  g.h = st[9 * N + c];
  g.n = st[10 * N + c];
  g.p = st[11 * N + c];
  g.xs = st[12 * N + c];
  g.k = st[13 * N + c];
  g.l = st[14 * N + c];
  v.Va = st[15 * N + c];
  g.ma = st[16 * N + c];
  g.ha = st[17 * N + c];
  g.xa = st[18 * N + c];
  const int k = steps[c];
  for (int j = 0; j < k; ++j) cell_step(P, v, g, 0.0f, 0.0f);
  st[0 * N + c] = v.Vd;
  st[1 * N + c] = g.r;
  st[2 * N + c] = g.s;
  st[3 * N + c] = g.q;
  st[4 * N + c] = (float)g.Ca;
  st[5 * N + c] = g.ICaH;
  st[7 * N + c] = v.Vs;
  st[8 * N + c] = g.m;
  st[9 * N + c] = g.h;
  st[10 * N + c] = g.n;
  st[11 * N + c] = g.p;
  st[12 * N + c] = g.xs;
  st[13 * N + c] = g.k;
  st[14 * N + c] = g.l;
  st[15 * N + c] = v.Va;
  st[16 * N + c] = g.ma;
  st[17 * N + c] = g.ha;
  st[18 * N + c] = g.xa;
}

}  // namespace
}  // namespace infoli

using namespace infoli;

#define CKI(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      if (d_st) cudaFree(d_st);                                                                    \
      if (d_steps) cudaFree(d_steps);                                                              \
      return infoli__fail(INFOLI_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));        \
    }                                                                                              \
  } while (0)

extern "C" int infoli_random_init(const float* params, int n, unsigned seed, float* state, int device) {
  infoli__clear_error();
  if (!params || !state || n <= 0) return infoli__fail(INFOLI_ERR_ARG, "random_init: bad argument");
  ModelParams P;
  std::memcpy(&P, params, sizeof P);
  // the reference's draws: g_CaL for every cell, then a step count per cell
  srand(seed);
  float* gcal = state + (size_t)INFOLI_S_G_CAL * n;
  for (int c = 0; c < n; ++c) gcal[c] = 0.6 + (0.2 * (rand() % 100) / 100);
  const int span = (int)std::ceil(100 / P.DELTA);
  std::vector<int> steps((size_t)n);
  for (int c = 0; c < n; ++c) steps[(size_t)c] = ((rand() % span) | 1) - 1;  // k drawn, k - 1 kept
  float* d_st = nullptr;
  int* d_steps = nullptr;
  CKI(cudaSetDevice(device));
  const size_t bytes = sizeof(float) * (size_t)INFOLI_NSTATE * n;
  CKI(cudaMalloc((void**)&d_st, bytes));
  CKI(cudaMalloc((void**)&d_steps, sizeof(int) * (size_t)n));
  CKI(cudaMemcpy(d_st, state, bytes, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(d_steps, steps.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
  isolated_steps_kernel<<<(n + 127) / 128, 128>>>(P, d_st, n, d_steps);
  CKI(cudaGetLastError());
  CKI(cudaMemcpy(state, d_st, bytes, cudaMemcpyDeviceToHost));
  cudaFree(d_st);
  cudaFree(d_steps);
  return INFOLI_OK;
}
