// msod_noalloc.cu -- element-table validation that allocates no device memory.
//
// msod_check_element_tables reports its verdict through a 4-byte device word
// that the library obtains with cudaMalloc on first use.  Some callers cannot
// let a library do that: a Fortran host whose device memory belongs to the
// OpenACC runtime's pool (a foreign cudaMalloc fragments or overcommits it),
// a process running under a capped or pre-reserved device allocator, or a
// program that must finish every allocation before it captures its work into
// a CUDA graph.  msod_check_element_tables_noalloc performs the same
// validation with its status word in the static device array below, so it
// calls no cudaMalloc, cudaFree or allocating library routine.
//
// The array is one 32-bit word (the stated maximum scratch of this entry
// point), is loaded with the library's device code on every GPU that uses the
// library and stays resident until the process exits.  Every call shares it
// and it keeps the last call's value, so each call clears it first; calls that
// overlap on the GPU (different streams, or different host threads on one
// device) race on the word and must be serialised by the caller.  Every call
// is synchronous (the verdict is copied back and the stream synchronised), so
// no call may be made on a capturing stream or during a global-mode capture.
#include <cuda_runtime.h>

#include <mutex>

#include "msod.h"
#include "msod_internal.h"
#include "msod_kernels.h"

namespace {

constexpr int kStatusWords = 1;
static __device__ __align__(256) int g_noalloc_status[kStatusWords];

std::mutex g_mu;
int *g_status_addr[64] = {nullptr};

// Device address of the status word for the current device.  Host code cannot
// use the symbol itself (it names a host-side stand-in), so the address is
// looked up once per device, with that device current, on the first call.
int status_address(int **out)
{
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return msod::set_error(MSOD_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(err));
    if (dev < 0 || dev >= 64) return msod::set_error(MSOD_ERR_NO_DEVICE, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_status_addr[dev]) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noalloc_status);
        if (err != cudaSuccess || !p)
            return msod::set_error(MSOD_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(err));
        g_status_addr[dev] = static_cast<int *>(p);
    }
    *out = g_status_addr[dev];
    return MSOD_OK;
}

int cuda_rc(cudaError_t err, const char *what)
{
    if (err == cudaSuccess) return MSOD_OK;
    return msod::set_error(MSOD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

}  // namespace

extern "C" int msod_check_element_tables_noalloc(int porder, int nelem, int npoin, const int *connec,
                                                 const float *dlxigp_ip, const int *invAtoIJK,
                                                 const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                                                 void *stream)
{
    msod::clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER)
        return msod::set_error(MSOD_ERR_PORDER, "porder %d outside 1..%d", porder, MSOD_MAX_PORDER);
    const long long n = (long long)(porder + 1) * (porder + 1) * (porder + 1);
    if (nelem < 1 || npoin < 1) return msod::set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    if ((long long)nelem * n >= (1LL << 31))
        return msod::set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode exceeds the int32 range of connec");
    if (!connec || !dlxigp_ip || !invAtoIJK || !gmshAtoI || !gmshAtoJ || !gmshAtoK)
        return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL table");
    int *word = nullptr;
    int rc = status_address(&word);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = cuda_rc(cudaMemsetAsync(word, 0, sizeof(int), st), "cudaMemsetAsync");
    if (rc) return rc;
    rc = cuda_rc(msod::launch_check_tables(porder, nelem, npoin, connec, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                                           gmshAtoK, word, st),
                 "check_tables launch");
    if (rc) return rc;
    int h = 0;
    rc = cuda_rc(cudaMemcpyAsync(&h, word, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    if (rc) return rc;
    rc = cuda_rc(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (rc) return rc;
    if (h)
        return msod::set_error(MSOD_ERR_BAD_TABLES,
                               "element tables failed validation (bits 0x%x: 1 invAtoIJK not a permutation, 2 "
                               "invAtoIJK/gmshAtoIJK disagree, 4 dlxigp_ip not 1-D structured, 8 connec out of range)",
                               h);
    return MSOD_OK;
}
