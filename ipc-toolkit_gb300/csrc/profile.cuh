// profile.cuh — per-kernel launch counting and CUDA-event timing.
//
// Every kernel of the library is launched through IPCG_LAUNCH.  Launches
// are always counted; when profiling is on, a CUDA event pair is recorded
// around the launch on its own stream and the elapsed time is accumulated
// per kernel name when the report is read.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace ipcg {
namespace prof {
bool enabled();
void count();
// a replayed CUDA graph launches `kernels` kernel nodes
void count_graph(int kernels);
void record(const char* name, cudaEvent_t a, cudaEvent_t b);
void make_events(cudaEvent_t* a, cudaEvent_t* b);
} // namespace prof
} // namespace ipcg

#define IPCG_LAUNCH(name, stream, ...)                                                                             \
    do {                                                                                                            \
        if (::ipcg::prof::enabled()) {                                                                              \
            cudaEvent_t a_, b_;                                                                                     \
            ::ipcg::prof::make_events(&a_, &b_);                                                                    \
            cudaEventRecord(a_, stream);                                                                            \
            __VA_ARGS__;                                                                                            \
            cudaEventRecord(b_, stream);                                                                            \
            ::ipcg::prof::record(name, a_, b_);                                                                     \
        } else {                                                                                                    \
            __VA_ARGS__;                                                                                            \
        }                                                                                                           \
        ::ipcg::prof::count();                                                                                      \
        IPCG_CHECK_LAUNCH();                                                                                        \
    } while (0)
