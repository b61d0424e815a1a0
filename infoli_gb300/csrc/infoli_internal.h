/* Internal helpers shared by the C and CUDA translation units of libinfoli_gpu.so. */
#ifndef INFOLI_INTERNAL_H
#define INFOLI_INTERNAL_H

#ifdef __cplusplus
extern "C" {
#endif

/* Record a message for infoli_last_error() and return `code`. */
int infoli__fail(int code, const char* fmt, ...)
#ifdef __GNUC__
    __attribute__((format(printf, 2, 3)))
#endif
    ;
void infoli__clear_error(void);

/* Limit of every bounded device-side wait, in ns: INFOLI_WAIT_TIMEOUT_MS
 * (default 4000 ms). */
unsigned long long infoli__wait_timeout_ns(void);

#ifdef __cplusplus
}

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

/* The library's stream-ordered device-memory pool of a device (release
 * threshold unlimited: freeing into it never unmaps memory, which would wait
 * for every kernel on the device). */
extern "C" cudaMemPool_t infoli__device_pool(int device);

/* Named NVTX range for the host phases (plan, upload, run, retire), so a
 * system profiler's timeline shows them; header-only, no library. */
struct InfoliRange {
  explicit InfoliRange(const char* name) { nvtxRangePushA(name); }
  ~InfoliRange() { nvtxRangePop(); }
  InfoliRange(const InfoliRange&) = delete;
  InfoliRange& operator=(const InfoliRange&) = delete;
};
#endif

#endif
