// colo_emu.cpp -- runtime of the host execution model (see shim/colo_emu.h).
// TEST INFRASTRUCTURE: used only to run the reference's sources on the CPU
// and record golden vectors.
#include "colo_emu.h"

#include <ucontext.h>

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
void (*colo_emu_hook_threshold)(const unsigned int*, unsigned int, unsigned int) = nullptr;
void (*colo_emu_hook_reduce)(size_t, unsigned long long) = nullptr;

namespace {
struct Fiber {
    ucontext_t ctx;
    bool done;
};
ucontext_t g_sched;
std::vector<Fiber> g_fibers;
std::vector<char> g_stacks;
const size_t kStack = 64 * 1024;
int g_cur = -1;
bool g_fiber_mode = false;
const std::function<void()>* g_body = nullptr;

void fiber_entry() {
    (*g_body)();
    g_fibers[g_cur].done = true;
}

struct Event {
    std::chrono::steady_clock::time_point t;
};
}  // namespace

void __syncthreads() {
    if (!g_fiber_mode) {
        std::fprintf(stderr, "colo_emu: __syncthreads in a kernel launched without barriers\n");
        std::abort();
    }
    swapcontext(&g_fibers[g_cur].ctx, &g_sched);
}

void colo_emu_launch(const char*, dim3 grid, dim3 block, bool barriers, const std::function<void()>& body) {
    gridDim = grid;
    blockDim = block;
    const unsigned nt = block.x * block.y * block.z;
    g_body = &body;
    if (barriers) {
        if (g_fibers.size() < nt) g_fibers.resize(nt);
        if (g_stacks.size() < nt * kStack) g_stacks.resize(nt * kStack);
    }
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = {bx, by, bz};
                if (!barriers) {
                    g_fiber_mode = false;
                    for (unsigned t = 0; t < nt; ++t) {
                        threadIdx = {t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
                        body();
                    }
                    continue;
                }
                g_fiber_mode = true;
                for (unsigned t = 0; t < nt; ++t) {
                    Fiber& f = g_fibers[t];
                    getcontext(&f.ctx);
                    f.ctx.uc_stack.ss_sp = g_stacks.data() + (size_t)t * kStack;
                    f.ctx.uc_stack.ss_size = kStack;
                    f.ctx.uc_link = &g_sched;
                    makecontext(&f.ctx, fiber_entry, 0);
                    f.done = false;
                }
                unsigned live = nt;
                while (live) {   // one round = every live thread runs to its next barrier
                    for (unsigned t = 0; t < nt; ++t) {
                        if (g_fibers[t].done) continue;
                        threadIdx = {t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
                        g_cur = (int)t;
                        swapcontext(&g_sched, &g_fibers[t].ctx);
                        if (g_fibers[t].done) live--;
                    }
                }
                g_fiber_mode = false;
            }
}

cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind k, cudaStream_t) {
    return cudaMemcpy(d, s, n, k);
}
cudaError_t cudaMemset(void* d, int v, size_t n) {
    if (n) std::memset(d, v, n);
    return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = (cudaEvent_t) new Event();
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t) {
    ((Event*)e)->t = std::chrono::steady_clock::now();
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = std::chrono::duration<float, std::milli>(((Event*)b)->t - ((Event*)a)->t).count();
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaGetLastError() { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "no error"; }
cudaError_t cudaDeviceReset() { return cudaSuccess; }
cudaError_t cudaGetDeviceCount(int* n) {
    *n = 1;
    return cudaSuccess;
}
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
    std::memset(p, 0, sizeof(*p));
    std::strcpy(p->name, "host emulation");
    p->major = 10;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
