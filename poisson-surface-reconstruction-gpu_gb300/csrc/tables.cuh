// Per-translation-unit copy of the constant look-up tables.  Each .cu file that includes
// this header owns one __constant__ copy and uploads it once per device through its
// upload function (see tables.cpp: fill_const_tables).
#pragma once
#include "psr_common.cuh"

namespace psr {

void fill_const_tables(ConstTables* t);   // host: derive the tables

}  // namespace psr

// c_tab (constant memory) serves warp-uniform indices; g_tab (global memory, read through
// the read-only cache) serves indices that differ between lanes (cube classes, edge and
// vertex kinds), which constant memory would serialise.
#define PSR_DEFINE_CONST_TABLES(upload_fn)                                          \
    namespace psr {                                                                 \
    static __constant__ ConstTables c_tab;                                          \
    static __device__ ConstTables g_tab;                                            \
    cudaError_t upload_fn() {                                                       \
        ConstTables t;                                                              \
        fill_const_tables(&t);                                                      \
        cudaError_t e = cudaMemcpyToSymbol(c_tab, &t, sizeof(ConstTables));         \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tab, &t, sizeof(ConstTables)); \
        return e;                                                                   \
    }                                                                               \
    }
