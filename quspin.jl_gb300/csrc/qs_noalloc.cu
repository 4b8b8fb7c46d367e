// qs_noalloc.cu -- host-buffer matvec that performs no device allocation.
//
// qs_op_matvec with host buffers stages x and y through device buffers that it
// allocates on first use.  Some callers cannot let a library allocate device
// memory: hosts whose device memory is owned by their own pool allocator with
// a hard limit (CUDA.jl and PyTorch keep a cache of their own, and a
// cudaMalloc behind its back can fail or force it to release its cache), and
// latency-bound loops that must not pay for cudaMalloc's implicit
// synchronisation.  This variant stages through one file-scope device array of
// fixed size instead, so a call allocates nothing.
//
// The array is shared by every call in the process and keeps the last call's
// contents; calls that overlap on the GPU (two host threads, or two streams)
// race on it and must be serialised by the caller.  The first call on each
// device looks up the array's device address (cudaGetSymbolAddress) with that
// device current; make that first call before any stream capture begins.
#include <cuda_runtime.h>

#include <mutex>

#include "qs_internal.h"

namespace qs {

namespace {

// Two staging vectors of kNoAllocVectorBytes each.
constexpr size_t kNoAllocVectorBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_stage[2 * kNoAllocVectorBytes];

std::mutex g_stage_mutex;
void* g_stage_addr[kMaxDevices] = {};

// Device address of the staging array on the current device (host code must
// not hand the symbol itself to a kernel: it names the host-side stand-in).
unsigned char* stage_address() {
    int dev = 0;
    QS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(QS_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_stage_mutex);
    if (!g_stage_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_stage);
        if (e != cudaSuccess || !p)
            throw Error(QS_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_stage_addr[dev] = p;
    }
    return static_cast<unsigned char*>(g_stage_addr[dev]);
}

}  // namespace

size_t noalloc_vector_bytes() { return kNoAllocVectorBytes; }

void op_matvec_noalloc(Op& op, int flags, cplx alpha, const void* x, int x_dtype, cplx beta, void* y, int y_dtype,
                       int64_t nrhs) {
    if (op.dense)
        throw Error(QS_ERR_UNSUPPORTED, "the allocation-free matvec covers orbit bases, not a sector from the dense "
                                        "nullspace intersection");
    const int64_t n = op.basis->n;
    auto bytes_of = [](int dt) -> size_t {
        switch (dt) {
            case QS_F64: return 8;
            case QS_C128: return 16;
            case QS_F32: return 4;
            case QS_C64: return 8;
            default: throw Error(QS_ERR_ARGUMENT, "unknown dtype");
        }
    };
    if (x_dtype != y_dtype)
        throw Error(QS_ERR_ARGUMENT, "the allocation-free matvec needs x and y of the same dtype");
    const bool ycx = (y_dtype == QS_C128 || y_dtype == QS_C64);
    if (!ycx && op.complex_mat) throw Error(QS_ERR_ARGUMENT, "the output must be complex for a complex operator");
    if (nrhs < 0) throw Error(QS_ERR_DIMENSION, "nrhs must be nonnegative");
    if (flags & ~(QS_TRANSPOSE | QS_CONJUGATE | QS_DOUBLE_FLOAT | QS_FIXED_POINT))
        throw Error(QS_ERR_ARGUMENT, "unknown flag bits");
    int dev = 0;
    QS_CUDA(cudaGetDevice(&dev));
    if (dev != op.device)
        throw Error(QS_ERR_ARGUMENT, "the operator lives on device " + std::to_string(op.device) +
                                         " but device " + std::to_string(dev) + " is current");
    const size_t vb = (size_t)n * bytes_of(y_dtype);
    if (vb > kNoAllocVectorBytes)
        throw Error(QS_ERR_ARGUMENT, "the allocation-free matvec stages at most " +
                                         std::to_string(kNoAllocVectorBytes >> 20) + " MiB per vector; this sector needs " +
                                         std::to_string(vb) + " bytes (use qs_op_matvec)");
    unsigned char* stage = stage_address();
    MatvecCall c;
    c.no_tune = true;   // variant timing would create events
    // the same flag meaning as qs_op_matvec: double-float products and
    // fixed-point row sums use tables and scratch that assembly allocated
    c.flags = flags & (QS_TRANSPOSE | QS_CONJUGATE);
    c.df = (flags & QS_DOUBLE_FLOAT) != 0;
    c.fx = (flags & QS_FIXED_POINT) != 0;
    c.alpha = alpha;
    c.beta = beta;
    c.single = (y_dtype == QS_F32 || y_dtype == QS_C64);
    c.x_complex = c.y_complex = ycx;
    c.x = stage;
    c.y = stage + kNoAllocVectorBytes;
    const bool beta_zero = beta.re == 0.0 && beta.im == 0.0;
    for (int64_t j = 0; j < nrhs; ++j) {
        QS_CUDA(cudaMemcpyAsync(stage, (const char*)x + (size_t)j * vb, vb, cudaMemcpyHostToDevice, op.stream));
        // with beta = 0 the kernels write every y entry without reading it, so
        // the previous call's contents never leak into the result
        if (!beta_zero)
            QS_CUDA(cudaMemcpyAsync(stage + kNoAllocVectorBytes, (const char*)y + (size_t)j * vb, vb,
                                    cudaMemcpyHostToDevice, op.stream));
        op_matvec_device(op, c, op.stream);
        QS_CUDA(cudaMemcpyAsync((char*)y + (size_t)j * vb, stage + kNoAllocVectorBytes, vb, cudaMemcpyDeviceToHost,
                                op.stream));
        QS_CUDA(cudaStreamSynchronize(op.stream));
    }
}

}  // namespace qs
