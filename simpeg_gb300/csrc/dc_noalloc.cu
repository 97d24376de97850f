// Allocation-free variant of the adjoint model-derivative entry point.
//
// dc_dadm_adj (dc_engine.cu) keeps its edge-product scratch (4 fp64 values per
// node) in buffers that its handle allocates with cudaMalloc on first use.
// Some callers cannot allocate device memory at that point: a host framework
// that has already reserved the GPU's memory for its own pool (an inversion
// server that pre-reserves HBM, a plugin host that forbids foreign
// allocations), or a caller that must not pay the implicit device
// synchronisation of cudaMalloc/cudaFree in the middle of its work.  For them
// dc_dadm_adj_noalloc runs the same two kernels with the scratch in a fixed
// file-scope device array and needs no handle: the caller passes the mesh
// widths, Robin face weights, inputs and output as device pointers.
//
// The array is sized for DC_NOALLOC_MAX_NODES nodes (4 doubles per node,
// 36.6 MiB) and every GPU that loads this library holds it until the process
// exits.  All calls share it and it keeps the previous call's contents; each
// call writes every entry it later reads (no clearing is needed), and calls
// that overlap on the GPU (e.g. on two streams) race on it.
#include "../../include/dcgpu.h"
#include "dc_internal.h"

#include <cstdio>

namespace dc {
namespace {

constexpr long long kMaxNodes = DC_NOALLOC_MAX_NODES;

// Edge products P (3 per node) and boundary products Q (1 per node).
static __device__ __align__(256) double g_noalloc_scratch[4 * kMaxNodes];

// Device address of g_noalloc_scratch on the current device.  In host code the
// symbol is only a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress, with the calling thread's device current.  It is looked
// up on every call (a table lookup in the runtime, no allocation): a cached
// address would go stale if the caller tore the context down
// (cudaDeviceReset) and the module were loaded again at another address.
int scratch_for_current_device(double **out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    last_error() = std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e);
    return DC_ERR_CUDA;
  }
  *out = static_cast<double *>(p);
  return DC_OK;
}

}  // namespace
}  // namespace dc

extern "C" int dc_dadm_adj_noalloc(int nx, int ny, int nz, const double *h_dev, const double *bface_dev,
                                   const double *u_dev, const double *lam_dev, int k, const double *dsig_dev,
                                   double scale, double *g_dev, void *stream) {
  using namespace dc;
  if (nx < 1 || ny < 1 || nz < 1 || k < 1 || !h_dev || !u_dev || !lam_dev || !g_dev) {
    last_error() = "dc_dadm_adj_noalloc: bad argument";
    return DC_ERR_ARG;
  }
  const long long N = (long long)(nx + 1) * (ny + 1) * (nz + 1);
  if (N > kMaxNodes) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "dc_dadm_adj_noalloc: mesh has %lld nodes, more than the no-allocation scratch holds (%lld); "
             "use dc_dadm_adj",
             N, kMaxNodes);
    last_error() = msg;
    return DC_ERR_ARG;
  }
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  // Geometry of the mesh as the kernels see it (no device allocation: the
  // caller's pointers are used directly; the host vectors stay empty).
  Level L;
  L.nx = nx;
  L.ny = ny;
  L.nz = nz;
  L.dims.Nx = nx + 1;
  L.dims.Ny = ny + 1;
  L.dims.Nz = nz + 1;
  L.dims.N = N;
  L.dims.mx = div_magic((unsigned)L.dims.Nx);
  L.dims.mxy = div_magic((unsigned)(L.dims.Nx * L.dims.Ny));
  L.d_h = const_cast<double *>(h_dev);
  L.d_bface = const_cast<double *>(bface_dev);
  const long long nyz = (long long)ny * nz, nxz = (long long)nx * nz, nxy = (long long)nx * ny;
  L.bface_off[0] = 0;
  L.bface_off[1] = nyz;
  L.bface_off[2] = 2 * nyz;
  L.bface_off[3] = 2 * nyz + nxz;
  L.bface_off[4] = 2 * nyz + 2 * nxz;
  L.bface_off[5] = 2 * nyz + 2 * nxz + nxy;
  L.bface_off[6] = 2 * nyz + 2 * nxz + 2 * nxy;
  cudaStream_t s = (cudaStream_t)stream;
  double *P = scratch;          // 3N
  double *Q = scratch + 3 * N;  // N
  edge_products(u_dev, lam_dev, k, L.dims, P, Q, s);
  cell_gradient(L, bface_dev != nullptr, P, Q, dsig_dev, scale, g_dev, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    last_error() = std::string("dc_dadm_adj_noalloc: ") + cudaGetErrorString(e);
    return DC_ERR_CUDA;
  }
  return DC_OK;
}
