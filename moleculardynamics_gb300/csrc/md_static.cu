// Bond-order forces without any device allocation (mdgb_many_body_forces_static).
//
// Some programs that call this library may not allocate GPU memory on their
// own: a host application that hands out all device memory from its own pool
// and forbids direct cudaMalloc/cudaFree (allocation behind its back breaks
// its memory budget), or a time-critical step loop that cannot afford the
// device-wide synchronisation cudaMalloc and cudaFree may cause.  The regular
// entry point mdgb_many_body_forces allocates its scratch on first use and
// grows it; this one keeps all of its scratch in one fixed array below that
// lives in the library's device image, so it never allocates.  The caller
// passes device arrays for the inputs and the output.
//
// Limits: at most kStaticMaxAtoms atoms and kStaticMaxSlots atom x row-slot
// pairs (n * nlargestsize).  The array is about 24 MB and every GPU that loads
// the library holds it until the process exits.  All calls share it and it
// keeps the last call's contents, so calls that overlap on the GPU (two
// streams, two host threads) race on it: serialise them.
#include <cstring>

#include "../../include/mdgb.h"
#include "md_forces.h"

using namespace mdgb;

namespace {

constexpr long long kStaticMaxAtoms = 16384;
constexpr long long kStaticMaxSlots = 1 << 20;

// layout: ell | short list (uint32 per slot), xsi | xsj (double per slot),
// len | slen (int per atom), flags (4 ints: missing count, ...)
constexpr size_t kOffEll = 0;
constexpr size_t kOffSl = kOffEll + 4 * kStaticMaxSlots;
constexpr size_t kOffXsi = kOffSl + 4 * kStaticMaxSlots;
constexpr size_t kOffXsj = kOffXsi + 8 * kStaticMaxSlots;
constexpr size_t kOffLen = kOffXsj + 8 * kStaticMaxSlots;
constexpr size_t kOffSlen = kOffLen + 4 * kStaticMaxAtoms;
constexpr size_t kOffFlags = kOffSlen + 4 * kStaticMaxAtoms;
constexpr size_t kStaticBytes = kOffFlags + 256;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// reference rows (i * nlistsize + k, -1 padded) -> ELL slot-major rows
__global__ void k_static_rows(const int* __restrict__ list, int n, int nlargest, int nls,
                              uint32_t* __restrict__ ell, int* __restrict__ len) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int* row = list + (size_t)i * nls;
  int k = 0;
  for (; k < nlargest && row[k] != -1; k++) ell[(size_t)k * n + i] = (uint32_t)row[k];
  len[i] = k;
}

void put_err(char* err, int err_len, const char* msg) {
  if (err && err_len > 0) {
    strncpy(err, msg, (size_t)err_len - 1);
    err[err_len - 1] = 0;
  }
}

}  // namespace

extern "C" int mdgb_many_body_forces_static(const double* d_pos4, double* d_f3, int n,
                                            int nlargestsize, int nlistsize,
                                            const int* d_list, double rcutsq, int ljexist,
                                            int* d_missing_xi, void* stream, char* err,
                                            int err_len) {
  if (n < 0 || nlistsize < 0 || nlargestsize < 0 || nlargestsize > nlistsize) {
    put_err(err, err_len, "bad size argument");
    return MD_BAD_ARGUMENT;
  }
  if (n == 0) return MD_OK;
  if (!d_pos4 || !d_f3 || (nlistsize > 0 && !d_list)) {
    put_err(err, err_len, "NULL device pointer");
    return MD_BAD_ARGUMENT;
  }
  if (((uintptr_t)d_pos4 & 31) != 0) {
    put_err(err, err_len, "positions must be 32-byte aligned (cudaMalloc memory is)");
    return MD_BAD_ARGUMENT;
  }
  const long long slots = (long long)n * (nlargestsize > 0 ? nlargestsize : 1);
  if (n > kStaticMaxAtoms || slots > kStaticMaxSlots) {
    put_err(err, err_len,
            "too large for the fixed scratch: at most 16384 atoms and 1048576 "
            "atom x row-slot pairs (n * nlargestsize)");
    return MD_BAD_ARGUMENT;
  }
  // The array's device address on the current device, looked up on every
  // call: the lookup allocates nothing, and an address kept from an earlier
  // call would be stale after the application reset the device (the
  // library's device image is then loaded again, possibly elsewhere).  The
  // first call on a device also loads that image.
  void* p = nullptr;
  cudaError_t e0 = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e0 != cudaSuccess || !p) {
    put_err(err, err_len, e0 != cudaSuccess ? cudaGetErrorString(e0) : "no device address");
    return e0 == cudaErrorNoDevice || e0 == cudaErrorInvalidDevice ? MD_NO_DEVICE
                                                                     : MD_CUDA_ERROR;
  }
  unsigned char* base = (unsigned char*)p;
  cudaStream_t st = (cudaStream_t)stream;
  int* flags = (int*)(base + kOffFlags);
  // only the missing-xi counter must start at zero; every other part of the
  // scratch is written before it is read within this call
  if (cudaMemsetAsync(flags, 0, 4 * sizeof(int), st) != cudaSuccess) {
    put_err(err, err_len, "cudaMemsetAsync failed");
    return MD_CUDA_ERROR;
  }
  uint32_t* ell = (uint32_t*)(base + kOffEll);
  int* len = (int*)(base + kOffLen);
  k_static_rows<<<(n + 127) / 128, 128, 0, st>>>(d_list, n, nlistsize ? nlargestsize : 0,
                                                 nlistsize, ell, len);
  MbArgs a{};
  a.pos = (const md_double4*)d_pos4;
  a.posf = nullptr;
  a.f3 = d_f3;
  a.n = n;
  a.list = ell;
  a.len = len;
  a.ld = n;
  a.grid = Grid{};
  a.cell3 = nullptr;
  a.ref_rows = d_list;
  a.ref_nls = nlistsize;
  a.ref_nlargest = nlistsize ? nlargestsize : 0;
  a.rcutsq = rcutsq;
  a.ljexist = ljexist;
  a.sl = (uint32_t*)(base + kOffSl);
  a.slen = (int*)(base + kOffSlen);
  a.xsi = base + kOffXsi;
  a.xsj = base + kOffXsj;
  a.missing = flags;
  launch_mb(a, false, false, st);
  // pass 2's count of xi reads that pass 1 never made (the regular entry
  // point reports it in its stats): copied on the caller's stream
  if (d_missing_xi &&
      cudaMemcpyAsync(d_missing_xi, flags, sizeof(int), cudaMemcpyDeviceToDevice, st) !=
          cudaSuccess) {
    put_err(err, err_len, "cudaMemcpyAsync failed");
    return MD_CUDA_ERROR;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    put_err(err, err_len, cudaGetErrorString(e));
    return MD_CUDA_ERROR;
  }
  return MD_OK;
}
