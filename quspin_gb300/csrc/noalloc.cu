// e^{aA} v with no device allocation: a fixed scratch area compiled into the
// library.
//
// Some callers of this library cannot allocate GPU memory themselves: a host
// application or plugin framework that reserves the device memory budget up
// front and hands out only the buffers it owns, or a tight time-stepping loop
// where cudaMalloc / cudaFree would synchronise the device between steps.
// qs_expm_multiply needs scratch beyond its inputs and outputs (two Taylor
// term buffers, the Taylor coefficients and the stopping-test control block);
// qs_expm_multiply_noalloc takes that scratch from the file-scope array below
// instead, so the caller passes only the matrix and the state.
//
// The array is static device memory: every GPU that loads libqsgpu.so holds it
// (QS_NOALLOC_BYTES, about 32 MiB) until the process exits, and every call
// shares it.  Consequently calls that overlap on the GPU (two streams, or two
// host threads) race on the same scratch and must be serialised by the
// caller.  The array keeps the last call's contents; each call re-zeroes the
// control block and rewrites the coefficients before it uses them.
#include "qs_common.cuh"
#include <complex>
#include <mutex>

// Largest state block n * nvec (complex128 elements) the scratch can hold.
#define QS_NOALLOC_MAX_ELEMS ((int64_t)1 << 20)
// Largest Taylor degree m* (the selection never exceeds 55).
#define QS_NOALLOC_MAX_TERMS 64

#define QS_NOALLOC_CTL_OFF 0                                    // control block, 256 B
#define QS_NOALLOC_COEFF_OFF 256                                // complex128[QS_NOALLOC_MAX_TERMS]
#define QS_NOALLOC_ETA_OFF (QS_NOALLOC_COEFF_OFF + 16 * QS_NOALLOC_MAX_TERMS)
#define QS_NOALLOC_ONE_OFF (QS_NOALLOC_ETA_OFF + 16)
#define QS_NOALLOC_WORK_OFF 2048                                // two complex128 buffers
#define QS_NOALLOC_BYTES (QS_NOALLOC_WORK_OFF + 2 * 16 * QS_NOALLOC_MAX_ELEMS)

static __device__ __align__(256) unsigned char g_noalloc_scratch[QS_NOALLOC_BYTES];

extern "C" int qs_expm_multiply(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                const void *data, int dtype, void *F, int64_t nvec, int s, int m_star, double tol,
                                double mu_re, double mu_im, const void *coeff, const void *eta, const void *one,
                                void *work, int btype, void *ctl, int group, void *stream);

// Writes the Taylor coefficients a / (s (j + 1)), eta and 1, and zeroes the
// control block, inside the scratch area.
__global__ void noalloc_prepare(unsigned char *scratch, double a_re, double a_im, int s, int m_star, double eta_re,
                                double eta_im)
{
    double *ctl = reinterpret_cast<double *>(scratch + QS_NOALLOC_CTL_OFF);
    cdbl *coeff = reinterpret_cast<cdbl *>(scratch + QS_NOALLOC_COEFF_OFF);
    for (int i = threadIdx.x; i < 32; i += blockDim.x) ctl[i] = 0.0;
    for (int j = threadIdx.x; j < QS_NOALLOC_MAX_TERMS; j += blockDim.x) {
        if (j < (m_star > 0 ? m_star : 1)) {
            double den = (double)s * (double)(j + 1);
            coeff[j] = cdbl{a_re / den, a_im / den};
        } else {
            coeff[j] = cdbl{0.0, 0.0};
        }
    }
    if (threadIdx.x == 0) {
        *reinterpret_cast<cdbl *>(scratch + QS_NOALLOC_ETA_OFF) = cdbl{eta_re, eta_im};
        *reinterpret_cast<cdbl *>(scratch + QS_NOALLOC_ONE_OFF) = cdbl{1.0, 0.0};
    }
}

#define QS_NOALLOC_MAX_DEVICES 64
static void *g_noalloc_ptr[QS_NOALLOC_MAX_DEVICES];
static cudaError_t g_noalloc_err[QS_NOALLOC_MAX_DEVICES];
static std::once_flag g_noalloc_once[QS_NOALLOC_MAX_DEVICES];

// Device address of the scratch array for the current device, looked up once
// per device with that device current (the first call on a device does this
// set-up; make that first call before capturing work on the stream).  The
// look-up runs under std::call_once, so host threads that make their first
// calls at the same time wait for one look-up.  The cached address belongs to
// the device's primary context: after cudaDeviceReset (or any reset of that
// context) reload the library before calling again.
static int noalloc_scratch(unsigned char **out)
{
    int dev = 0;
    QS_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= QS_NOALLOC_MAX_DEVICES) return QS_ERR_UNSUPPORTED;
    std::call_once(g_noalloc_once[dev], [dev] {
        void *p = nullptr;
        g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        g_noalloc_ptr[dev] = g_noalloc_err[dev] == cudaSuccess ? p : nullptr;
    });
    if (g_noalloc_err[dev] != cudaSuccess || !g_noalloc_ptr[dev]) return QS_ERR_CUDA;
    *out = reinterpret_cast<unsigned char *>(g_noalloc_ptr[dev]);
    return QS_OK;
}

extern "C" int64_t qs_expm_noalloc_max_elems() { return QS_NOALLOC_MAX_ELEMS; }

// In-place e^{aA} F for a CSR matrix A (values dtype QS_F64 or QS_C128) and
// a complex128 state block F[n, nvec], with s substeps of at most m_star
// Taylor terms, tolerance tol and shift mu: the arithmetic of
// qs_expm_multiply with complex128 Taylor buffers, but every scratch buffer
// taken from the library's static array.  Returns QS_ERR_CAPACITY (-5) when
// n * nvec exceeds qs_expm_noalloc_max_elems() (1,048,576) or m_star exceeds
// 64.  Calls no cudaMalloc / cudaFree.
extern "C" int qs_expm_multiply_noalloc(int64_t n, int64_t nnz, const void *indptr, int idx64,
                                        const int32_t *indices, const void *data, int dtype, void *F, int64_t nvec,
                                        int s, int m_star, double tol, double mu_re, double mu_im, double a_re,
                                        double a_im, int group, void *stream)
{
    if (n < 1 || nvec < 1 || s < 1 || m_star < 0 || !indptr || !F) return QS_ERR_ARG;
    if (dtype != QS_F64 && dtype != QS_C128) return QS_ERR_ARG;
    if (n > QS_NOALLOC_MAX_ELEMS || nvec > QS_NOALLOC_MAX_ELEMS || n * nvec > QS_NOALLOC_MAX_ELEMS) return QS_ERR_CAPACITY;
    if (m_star > QS_NOALLOC_MAX_TERMS) return QS_ERR_CAPACITY;
    unsigned char *scr = nullptr;
    int rc = noalloc_scratch(&scr);
    if (rc) return rc;
    const std::complex<double> a(a_re, a_im), mu(mu_re, mu_im);
    const std::complex<double> eta = std::exp(a * mu / (double)s);
    cudaStream_t st = qs_stream(stream);
    noalloc_prepare<<<1, 64, 0, st>>>(scr, a_re, a_im, s, m_star, eta.real(), eta.imag());
    QS_CHECK(cudaGetLastError());
    return qs_expm_multiply(n, nnz, indptr, idx64, indices, data, dtype, F, nvec, s, m_star, tol, mu_re, mu_im,
                            scr + QS_NOALLOC_COEFF_OFF, scr + QS_NOALLOC_ETA_OFF, scr + QS_NOALLOC_ONE_OFF,
                            scr + QS_NOALLOC_WORK_OFF, QS_C128, scr + QS_NOALLOC_CTL_OFF, group, stream);
}
