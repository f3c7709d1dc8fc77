// Per-translation-unit copy of the constant look-up tables.  Each .cu file that includes
// this header owns one __constant__ copy and uploads it once per device through its
// upload function (see tables.cpp: fill_const_tables).
#pragma once
#include "psr_common.cuh"

namespace psr {

void fill_const_tables(ConstTables* t);   // host: derive the tables

}  // namespace psr

#define PSR_DEFINE_CONST_TABLES(upload_fn)                                          \
    namespace psr {                                                                 \
    static __constant__ ConstTables c_tab;                                          \
    cudaError_t upload_fn() {                                                       \
        ConstTables t;                                                              \
        fill_const_tables(&t);                                                      \
        return cudaMemcpyToSymbol(c_tab, &t, sizeof(ConstTables));                  \
    }                                                                               \
    }
