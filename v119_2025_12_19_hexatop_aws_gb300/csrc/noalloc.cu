// hexa_filter_noalloc: the Helmholtz density filter of hexa_filter for callers
// that cannot allocate device memory.
//
// Some callers must not call cudaMalloc (or any allocating routine) at the
// point where they filter: code that runs on its own stream while another
// stream of the application is being captured into a CUDA graph (during a
// global-mode capture an allocation is a prohibited call on every thread), or
// hosts that hand the whole device-memory budget to their own pool and forbid
// other allocations mid-run.  This entry point takes device arrays for its
// input and output and keeps all of its scratch -- the six work vectors and
// the inverse diagonal of the Jacobi-PCG, the reduction partials, the ticket
// counter and the iteration scalars -- in one file-scope device array of fixed
// size, so it allocates nothing: no cudaMalloc, no cudaFree, no allocating
// library call.
//
// The call itself cannot be captured: it reads the iteration scalars back to
// the host between groups of iterations and synchronizes its stream.  The
// stream it is given must therefore not be capturing (HEXA_ERR_ARG
// otherwise).  While another stream captures, pass a non-blocking stream
// (cudaStreamNonBlocking): work on the legacy default stream (stream NULL)
// would join a capture on any blocking stream.  For its own duration the call
// switches the calling thread to the relaxed capture mode
// (cudaThreadExchangeStreamCaptureMode), so its copies and synchronizations are
// not refused because the application is capturing elsewhere, and restores the
// thread's mode before it returns.
//
// The array holds HEXA_NOALLOC_MAX_NODES grid nodes (about 15 MB); every GPU
// that loads the library keeps it until the process exits.  Every call shares
// it and it keeps the last call's contents, so each call clears what must
// start at zero (the ticket counter) and rewrites everything else before use;
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on the array and must be serialised by the
// caller.  The first call on each device resolves the array's device address
// with cudaGetSymbolAddress (under a lock, with that device current); make
// that first call before any stream capture begins.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>

#include "../../include/hexagpu.h"
#include "element.h"
#include "hexa_kernels.h"

namespace {

using namespace hexa;

constexpr long long kMaxNodes = HEXA_NOALLOC_MAX_NODES;
constexpr int kVecs = 7;                // b, x, r, z, p, q, dinv
constexpr long long kHeader = 4224;      // doubles: scalars, ticket, results, partials
constexpr long long kScratchDoubles = kHeader + kVecs * kMaxNodes;
constexpr int kRedBlocksNA = 152 * 4;    // grid of the reducing vector passes
constexpr int kMaxDevices = 64;

// The scratch.  In host code this name is a host-side stand-in, never a device
// address: kernels receive the address cudaGetSymbolAddress returns.
static __device__ __align__(256) double g_filter_scratch[kScratchDoubles];

std::mutex g_lock;
double* g_addr[kMaxDevices] = {nullptr};

double* scratch_for_current_device(int* err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    *err = HEXA_ERR_NO_DEVICE;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_lock);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_filter_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      *err = HEXA_ERR_CUDA;
      return nullptr;
    }
    g_addr[dev] = (double*)p;
  }
  return g_addr[dev];
}

// Device memory of the current device (or managed memory): anything else --
// host memory, or an array on another GPU while the scratch is resolved for
// the current one -- is rejected.
bool on_current_device(const void* p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  if (a.type != cudaMemoryTypeDevice) return false;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.device == dev;
}

// Restores the calling thread's stream-capture mode on every return path.
struct RelaxedCaptureMode {
  cudaStreamCaptureMode prev = cudaStreamCaptureModeRelaxed;
  bool ok = false;
  RelaxedCaptureMode() { ok = cudaThreadExchangeStreamCaptureMode(&prev) == cudaSuccess; }
  ~RelaxedCaptureMode() {
    if (ok) cudaThreadExchangeStreamCaptureMode(&prev);
  }
};

}  // namespace

extern "C" int hexa_filter_noalloc(const hexa_grid* g, const double* rho_in, double radius, double tol,
                                   int32_t max_iter, int32_t quirk, double* rho_out, void* stream,
                                   hexa_filter_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!g || g->nx < 1 || g->ny < 1 || g->nz < 1 || !(g->dx > 0 && g->dy > 0 && g->dz > 0) || !(radius >= 0) ||
      !(tol > 0) || max_iter < 1)
    return HEXA_ERR_ARG;
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  if (G.nnode() > kMaxNodes) return HEXA_ERR_TOO_LARGE;
  RelaxedCaptureMode relaxed;  // before any other CUDA call of this entry point
  if (!relaxed.ok) {
    cudaGetLastError();
    return HEXA_ERR_CUDA;
  }
  // staging a host array would need an allocation
  if (!on_current_device(rho_in) || !on_current_device(rho_out)) return HEXA_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (st) {  // the call synchronizes: it cannot run on a stream that is being captured
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
      cudaGetLastError();
      return HEXA_ERR_ARG;
    }
    if (cs != cudaStreamCaptureStatusNone) return HEXA_ERR_ARG;
  }
  int err = 0;
  double* base = scratch_for_current_device(&err);
  if (!base) return err;

  double Ke[64], Me[64];
  if (scalar_matrices(g->dx, g->dy, g->dz, quirk, Ke, Me) != 0) return HEXA_ERR_ARG;
  HelmK K;
  helm_corner_matrix(Ke, Me, radius, K.A);
  K.rhs_scale = g->dx * g->dy * g->dz / 8.0;

  PcgScalars* s = (PcgScalars*)base;
  unsigned* ticket = (unsigned*)(base + 64);
  double* result = base + 96;
  double* partials = base + 128;
  const long long nn = G.nnode();
  double* vec = base + kHeader;
  double *b = vec, *x = vec + kMaxNodes, *r = vec + 2 * kMaxNodes, *z = vec + 3 * kMaxNodes,
         *p = vec + 4 * kMaxNodes, *q = vec + 5 * kMaxNodes, *dinv = vec + 6 * kMaxNodes;

  // the previous call's contents stay behind: the ticket must start at zero
  cudaMemsetAsync(ticket, 0, sizeof(unsigned), st);
  launch_helm_rhs<double>(G, rho_in, K.rhs_scale, b, st);
  launch_helm_dinv<double>(G, K, dinv, st);
  RedArgs rd;
  rd.partials = partials;
  rd.ticket = ticket;
  rd.s = s;
  rd.dst = result;
  rd.op = FIN_STORE;
  rd.nsum = 1;
  launch_dot<double>(b, b, (const double*)nullptr, (const double*)nullptr, nn, rd, kRedBlocksNA, nullptr, st);
  double bb = 0.0;
  cudaMemcpyAsync(&bb, result, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return HEXA_ERR_CUDA;
  }
  hexa_filter_stats out;
  std::memset(&out, 0, sizeof(out));
  const double bnorm = std::sqrt(bb);
  if (bnorm == 0.0) {  // GPUHelmholtz.jl:203-206: the input comes back unchanged
    cudaMemcpyAsync(rho_out, rho_in, sizeof(double) * G.nelem(), cudaMemcpyDeviceToDevice, st);
  } else {
    PcgScalars hs;
    std::memset(&hs, 0, sizeof(hs));
    hs.tol = tol;
    hs.max_iter = max_iter;
    hs.cadence = -10;
    hs.no_div = 1;
    hs.bnorm = bnorm;
    hs.best_rel = INFINITY;
    cudaMemcpyAsync(s, &hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, st);
    launch_fill<double>(x, 0.0, nn, st);
    launch_copy<double>(r, b, nn, st);
    rd.op = FIN_INIT_RZ;
    launch_jacobi_precond<double>(z, r, dinv, nn, rd, kRedBlocksNA, nullptr, st);
    launch_copy<double>(p, z, nn, st);
    const int hblocks = (int)std::min<long long>((nn + 255) / 256, 152 * 8);
    for (int guard = 0; guard <= max_iter / 10 + 1; ++guard) {
      for (int it = 0; it < 10; ++it) {
        RedArgs ra = rd;
        ra.op = FIN_PCG_ALPHA;
        launch_helm_apply_dot<double>(G, K, p, q, ra, hblocks, &s->halt, st);
        RedArgs rb = rd;
        rb.op = FIN_PCG_RES;
        rb.nsum = 2;
        launch_pcg_update<double>(x, r, z, p, q, dinv, nn, rb, kRedBlocksNA, s, st);
        launch_p_update<double>(p, z, nn, s, st);
      }
      cudaMemcpyAsync(&hs, s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return HEXA_ERR_CUDA;
      }
      if (hs.halt) break;
    }
    if (hs.status == 2 || hs.status == 4) {
      // a NaN residual or a breakdown of p.Ap gives a NaN field, as hexa_filter
      // and the reference's loop do (its callers test for it, TopOpt.jl:360-363)
      launch_fill<double>(rho_out, std::numeric_limits<double>::quiet_NaN(), G.nelem(), st);
    } else {
      launch_helm_extract<double>(G, x, rho_out, st);
    }
    out.iterations = hs.iter;
    out.relres = hs.relres;
  }
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return HEXA_ERR_CUDA;
  out.status = HEXA_OK;
  out.solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = out;
  return HEXA_OK;
}
