/* Test helper, preloaded (LD_PRELOAD) into a child process by
 * tests/test_zz_no_alloc.py: it counts the CUDA runtime calls that allocate
 * or free memory or create streams, events or graphs, and forwards each to
 * the real runtime. esf_test_alloc_calls() returns the count so far, so a
 * test can show that a call made none of them, even an allocation freed
 * again before the call returns. Not part of the library. */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stddef.h>

typedef int cuda_error;
static unsigned long long g_calls;

unsigned long long esf_test_alloc_calls(void) {
  return __atomic_load_n(&g_calls, __ATOMIC_RELAXED);
}

#define FORWARD(name, params, args)                                   \
  cuda_error name params {                                            \
    static cuda_error(*real) params;                                  \
    if (!real) *(void**)(&real) = dlsym(RTLD_NEXT, #name);            \
    __atomic_add_fetch(&g_calls, 1, __ATOMIC_RELAXED);                \
    return real ? real args : 999; /* 999: cudaErrorUnknown */        \
  }

FORWARD(cudaMalloc, (void** p, size_t n), (p, n))
FORWARD(cudaFree, (void* p), (p))
FORWARD(cudaMallocAsync, (void** p, size_t n, void* s), (p, n, s))
FORWARD(cudaFreeAsync, (void* p, void* s), (p, s))
FORWARD(cudaMallocHost, (void** p, size_t n), (p, n))
FORWARD(cudaHostAlloc, (void** p, size_t n, unsigned f), (p, n, f))
FORWARD(cudaFreeHost, (void* p), (p))
FORWARD(cudaMallocManaged, (void** p, size_t n, unsigned f), (p, n, f))
FORWARD(cudaMallocPitch, (void** p, size_t* pitch, size_t w, size_t h), (p, pitch, w, h))
FORWARD(cudaStreamCreate, (void** s), (s))
FORWARD(cudaStreamCreateWithFlags, (void** s, unsigned f), (s, f))
FORWARD(cudaStreamCreateWithPriority, (void** s, unsigned f, int prio), (s, f, prio))
FORWARD(cudaEventCreate, (void** e), (e))
FORWARD(cudaEventCreateWithFlags, (void** e, unsigned f), (e, f))
FORWARD(cudaGraphInstantiate, (void** e, void* g, unsigned long long f), (e, g, f))
FORWARD(cudaStreamBeginCapture, (void* s, int mode), (s, mode))
