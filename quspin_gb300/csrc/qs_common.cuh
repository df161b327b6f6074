// Common definitions for the GB300 hot-path library (libqsgpu.so).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define QS_OK 0
#define QS_ERR_ARG -1        // invalid argument (sizes, pointers, enums)
#define QS_ERR_CUDA -2       // a CUDA runtime call failed
#define QS_ERR_OPSTR -3      // unknown operator character
#define QS_ERR_COMPLEX -4    // complex matrix element requested in a real dtype
#define QS_ERR_CAPACITY -5   // output buffer too small
#define QS_ERR_UNSUPPORTED -6
#define QS_ERR_NOT_CONVERGED -7

// value / vector element types shared with the Python side
#define QS_F32 0
#define QS_F64 1
#define QS_C64 2
#define QS_C128 3
#define QS_PF 4        // real value kept as a pair of floats hi + lo (8 bytes)
#define QS_CPF 5       // complex value kept as two float pairs {re.hi, re.lo, im.hi, im.lo} (16 bytes)
#define QS_PF8 6       // real float-pair values as codes: QS_CODE_TABLE pairs, then one uint8 code per nonzero
#define QS_CPF8 7      // complex float-pair values as codes: QS_CODE_TABLE complex pairs, then one uint8 code each
#define QS_PF8P 8      // QS_PF8 with each code byte packed into the low 8 bits of its column word (col << 8 | code;
                       // data holds only the table); single-vector Taylor terms and the SpMV, n < 2^23
#define QS_CPF8P 9     // the same for QS_CPF8
#define QS_CODE_TABLE 256

#define QS_CHECK(call)                                   \
    do {                                                 \
        cudaError_t e__ = (call);                        \
        if (e__ != cudaSuccess) return QS_ERR_CUDA;      \
    } while (0)

static inline cudaStream_t qs_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

static inline int qs_num_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

// Blocks of a grid-stride kernel that are resident on all SMs at once
// (its occupancy at `threads` threads and no dynamic shared memory), at most
// `need` and at least 1.  `cache` keeps the per-SM count between calls (one
// cache per kernel instantiation: a function-local static at the call site).
template <class K>
static inline int qs_persistent_grid(K kern, int threads, int64_t need, int &cache)
{
    if (cache <= 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, threads, 0) != cudaSuccess || b < 1) b = 1;
        cache = b;
    }
    const int64_t cap = (int64_t)qs_num_sms() * cache;
    return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

// complex helpers (plain structs; no std::complex in device code)
struct cdbl { double x, y; };
struct cflt { float x, y; };

template <typename T> struct is_cplx { static constexpr bool value = false; };
template <> struct is_cplx<cdbl> { static constexpr bool value = true; };
template <> struct is_cplx<cflt> { static constexpr bool value = true; };
