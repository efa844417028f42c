// extern "C" entry points of libhexagpu.so (declared in include/hexagpu.h).
//
// Every array argument may be a host pointer (pageable or pinned) or a
// device pointer; host arrays are staged through the context's cached device
// buffers, device arrays are used in place.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <vector>

#include "element.h"
#include "hexa_kernels.h"
#include "solver.h"

using namespace hexa;

struct hexa_ctx {
  Ctx c;
};

namespace {

constexpr int kRed = 152 * 4;

int set_err(hexa_ctx* h, int code, const std::string& msg) {
  if (h) h->c.err = msg;
  return code;
}

bool valid_grid(const hexa_grid* g) {
  return g && g->nx >= 1 && g->ny >= 1 && g->nz >= 1 && g->dx > 0 && g->dy > 0 && g->dz > 0 &&
         (long long)(g->nx + 1) * (g->ny + 1) * (g->nz + 1) * 3LL < (1LL << 40);
}

// Device view of an input array: the pointer itself when it is on the
// device, else a cached staging buffer filled by an async H2D copy.
template <typename T>
const T* stage_in(Ctx& c, const T* p, size_t n, const char* name) {
  if (!p) return nullptr;
  if (is_device_ptr(p)) return p;
  T* d = c.vec<T>(name, n);
  if (!d) return nullptr;
  cudaMemcpyAsync(d, p, n * sizeof(T), cudaMemcpyHostToDevice, c.st);
  return d;
}

template <typename T>
T* out_buf(Ctx& c, T* p, size_t n, const char* name) {
  if (is_device_ptr(p)) return p;
  return c.vec<T>(name, n);
}

template <typename T>
void stage_out(Ctx& c, T* user, const T* dev, size_t n) {
  if (user != dev) cudaMemcpyAsync(user, dev, n * sizeof(T), cudaMemcpyDeviceToHost, c.st);
}

// Per-node fixed bits from a per-DOF byte mask (host or device).
const uint8_t* node_mask(Ctx& c, const Grid& g, const uint8_t* fixed_dof) {
  if (!fixed_dof) return nullptr;
  const long long nn = g.nnode();
  std::vector<uint8_t> host(3 * nn);
  if (is_device_ptr(fixed_dof)) {
    cudaMemcpyAsync(host.data(), fixed_dof, 3 * nn, cudaMemcpyDeviceToHost, c.st);
    cudaStreamSynchronize(c.st);
  } else {
    std::memcpy(host.data(), fixed_dof, 3 * nn);
  }
  std::vector<uint8_t> bits(nn);
  bool any = false;
  for (long long n = 0; n < nn; ++n) {
    const uint8_t b = (host[3 * n] ? 1 : 0) | (host[3 * n + 1] ? 2 : 0) | (host[3 * n + 2] ? 4 : 0);
    bits[n] = b;
    any |= (b != 0);
  }
  if (!any) return nullptr;
  uint8_t* d = c.vec<uint8_t>("nodemask", nn);
  if (!d) return nullptr;
  cudaMemcpyAsync(d, bits.data(), nn, cudaMemcpyHostToDevice, c.st);
  cudaStreamSynchronize(c.st);  // bits is a local vector
  return d;
}

bool prepare_problem(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, const double* factor,
                     const double* f, Problem* P) {
  Ctx& c = h->c;
  P->g = make_grid(g->nx, g->ny, g->nz);
  P->dx = g->dx;
  P->dy = g->dy;
  P->dz = g->dz;
  P->nu = nu;
  P->m.faces = bc ? bc->clamp_faces : 0u;
  P->m.node = bc ? node_mask(c, P->g, bc->fixed_dof) : nullptr;
  if (bc && bc->fixed_dof && !c.err.empty()) return false;
  P->fac64 = stage_in<double>(c, factor, P->g.nelem(), "in_factor");
  if (!P->fac64) return false;
  if (f) {
    const double* fr = stage_in<double>(c, f, P->g.ndof(), "in_f_raw");
    double* fm = c.vec<double>("in_f", P->g.ndof());
    if (!fr || !fm) return false;
    launch_mask_copy<double, double>(P->g, P->m, fm, fr, c.st);
    c.launches++;
    P->f64 = fm;
  } else {
    P->f64 = nullptr;
  }
  return true;
}

// A staged operator launch that gave up a bounded wait (op.cu) leaves its
// output incomplete: the call reports it as a CUDA-level failure.
bool staging_ok(hexa_ctx* h, const char* where) {
  if (!op_take_wait_error(h->c.st)) return true;
  h->c.err = std::string(where) + ": an operator launch gave up waiting for its staged input (bounded wait ran out)";
  return false;
}

double wall_ms(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

int hexa_version(void) { return 100; }

void hexa_default_params(hexa_solve_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->nu = 0.3;
  p->tol = 1e-9;
  p->max_iter = 30000;          // configs/default.yaml:222
  p->precond = HEXA_PRECOND_MULTIGRID;
  p->shift_factor = 1e-10;      // H100/H200/A100 profile (src/Main.jl:108)
  p->stagnation_tol = 0.0;
  p->max_shift_attempts = 3;    // GPUSolver.jl:217 default
  p->shift_multiplier = 10.0;   // GPUSolver.jl:218 default
  p->check_cadence = 1;
  p->diag_quirk = 1;
  p->precision = HEXA_PREC_FP64;
  p->mg_levels = 0;
  p->pre_smooth = 2;
  p->post_smooth = 2;
  p->smoother = HEXA_SMOOTH_CHEBYSHEV;
  p->jacobi_omega = 0.0;        // 0: 1.2 / (element bound on lambda_max(D^-1 A))
  p->cheb_ratio = 10;
  p->coarse_iters = 30;
  p->inner_tol = 1e-4;
  p->max_outer = 20;
  p->use_graphs = 1;
  p->graph_iters = 10;
  p->true_residual = 1;
  p->divergence_check = 1;
  p->autotune = 0;
  p->mg_cycle = 1;
}

int hexa_create(int32_t device, hexa_ctx** out) {
  if (!out) return HEXA_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return HEXA_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return HEXA_ERR_ARG;
  hexa_ctx* h = new (std::nothrow) hexa_ctx();
  if (!h) return HEXA_ERR_NOMEM;
  Ctx& c = h->c;
  c.device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return HEXA_ERR_CUDA;
  }
  for (auto& e : c.ev) cudaEventCreate(&e);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = ~0ULL;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  c.ticket = c.vec<unsigned>("ticket", 64);  // [0, 16): per-column reductions, 32: gram
  c.s = c.vec<PcgScalars>("scalars", 1);
  c.s2 = c.vec<PcgScalars>("scalars2", 1);
  c.dscal = c.vec<double>("dscal", 64);
  if (!c.ticket || !c.s || !c.s2 || !c.dscal || !c.ensure_partials(1 << 16)) {
    hexa_destroy(h);
    return HEXA_ERR_NOMEM;
  }
  cudaMemsetAsync(c.ticket, 0, 64 * sizeof(unsigned), c.st);
  cudaMemsetAsync(c.s, 0, sizeof(PcgScalars), c.st);
  cudaMemsetAsync(c.s2, 0, sizeof(PcgScalars), c.st);
  if (cudaMallocHost(&c.hs, sizeof(PcgScalars)) != cudaSuccess || cudaMallocHost(&c.hscal, 64 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    hexa_destroy(h);
    return HEXA_ERR_NOMEM;
  }
  if (cudaStreamSynchronize(c.st) != cudaSuccess) {
    cudaGetLastError();
    hexa_destroy(h);
    return HEXA_ERR_CUDA;
  }
  *out = h;
  return HEXA_OK;
}

void hexa_destroy(hexa_ctx* h) {
  if (!h) return;
  Ctx& c = h->c;
  cudaSetDevice(c.device);
  if (c.st) cudaStreamSynchronize(c.st);
  for (auto& kv : c.bufs) cudaFreeAsync(kv.second.first, c.st);
  c.bufs.clear();
  if (c.st) {
    cudaStreamSynchronize(c.st);
    cudaStreamDestroy(c.st);
  }
  for (auto& e : c.ev)
    if (e) cudaEventDestroy(e);
  if (c.hs) cudaFreeHost(c.hs);
  if (c.hscal) cudaFreeHost(c.hscal);
  cudaGetLastError();
  delete h;
}

const char* hexa_last_error(const hexa_ctx* h) { return h ? h->c.err.c_str() : "null context"; }
double hexa_last_device_ms(const hexa_ctx* h) { return h ? h->c.last_ms : 0.0; }
int64_t hexa_kernel_launches(const hexa_ctx* h) { return h ? h->c.launches : 0; }

int hexa_canonical_stiffness(double dx, double dy, double dz, double nu, double* ke_out) {
  if (!ke_out) return HEXA_ERR_ARG;
  return canonical_stiffness(dx, dy, dz, nu, ke_out) == 0 ? HEXA_OK : HEXA_ERR_ARG;
}

int hexa_scalar_canonical_matrices(double dx, double dy, double dz, int32_t quirk, double* ke_out, double* me_out) {
  if (!ke_out || !me_out) return HEXA_ERR_ARG;
  return scalar_matrices(dx, dy, dz, quirk, ke_out, me_out) == 0 ? HEXA_OK : HEXA_ERR_ARG;
}

}  // extern "C"

template <typename T>
static int apply_operator_t(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, const T* factor,
                            const T* x, T sigma, T* y) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !factor || !x || !y) return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  ModalK<double> K64;
  std::string e;
  if (!build_modal(g->dx, g->dy, g->dz, nu, &K64, &e)) return set_err(h, HEXA_ERR_ARG, e);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  Mask m;
  m.faces = bc ? bc->clamp_faces : 0u;
  m.node = bc ? node_mask(c, G, bc->fixed_dof) : nullptr;
  const T* fac = stage_in<T>(c, factor, G.nelem(), sizeof(T) == 8 ? "ap_fac64" : "ap_fac32");
  const T* xr = stage_in<T>(c, x, G.ndof(), sizeof(T) == 8 ? "ap_xr64" : "ap_xr32");
  T* xm = c.vec<T>(sizeof(T) == 8 ? "ap_x64" : "ap_x32", G.ndof());
  T* yd = out_buf<T>(c, y, G.ndof(), sizeof(T) == 8 ? "ap_y64" : "ap_y32");
  if (!fac || !xr || !xm || !yd) return HEXA_ERR_NOMEM;
  launch_mask_copy<T, T>(G, m, xm, xr, c.st);
  OpArgs<T> a;
  a.g = G;
  a.m = m;
  a.x = xm;
  a.fac = fac;
  a.b = nullptr;
  a.y = yd;
  if constexpr (sizeof(T) == 8) a.K = K64;
  else a.K = modal_to_f32(K64);
  a.sigma = sigma;
  a.omega = T(0);
  a.kchunk = op_pick_kchunk<T>(G);
  a.diag_quirk = 0;
  a.xin = nullptr;
  a.c1 = a.c2 = T(0);
  a.red.partials = c.partials;
  a.red.ticket = c.ticket;
  a.red.dst = nullptr;
  a.red.s = nullptr;
  a.red.op = FIN_NONE;
  a.red.nsum = 1;
  a.halt = nullptr;
  cudaEventRecord(c.ev[0], c.st);
  launch_op<T>(OP_APPLY, a, c.st);
  cudaEventRecord(c.ev[1], c.st);
  c.launches += 2;
  stage_out<T>(c, y, yd, G.ndof());
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("apply")) return set_err(h, HEXA_ERR_CUDA, c.err);
  if (!staging_ok(h, "apply")) return HEXA_ERR_CUDA;
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]);
  c.last_ms = ms;
  return HEXA_OK;
}


extern "C" {

int hexa_apply_operator(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, const double* factor,
                        const double* x, double sigma, double* y) {
  return apply_operator_t<double>(h, g, bc, nu, factor, x, sigma, y);
}

int hexa_apply_operator_f32(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, const float* factor,
                            const float* x, float sigma, float* y) {
  return apply_operator_t<float>(h, g, bc, nu, factor, x, sigma, y);
}

}  // extern "C"

template <typename T>
static int time_operator_t(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, int mode, const T* factor,
                           const T* x, const T* b, T* y, int reps, double* avg_ms) {
  Ctx& c = h->c;
  ModalK<double> K64;
  std::string e;
  if (!build_modal(g->dx, g->dy, g->dz, nu, &K64, &e)) return set_err(h, HEXA_ERR_ARG, e);
  if (!is_device_ptr(factor) || !is_device_ptr(x) || !is_device_ptr(y) || (b && !is_device_ptr(b)))
    return set_err(h, HEXA_ERR_ARG, "hexa_time_operator takes device arrays");
  if ((mode == OP_RESID || mode == OP_JACOBI || mode == OP_CHEB2) && !b) return set_err(h, HEXA_ERR_ARG, "mode needs b");
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  Mask m;
  m.faces = bc ? bc->clamp_faces : 0u;
  m.node = bc ? node_mask(c, G, bc->fixed_dof) : nullptr;
  OpArgs<T> a;
  a.g = G;
  a.m = m;
  a.x = x;
  a.fac = factor;
  a.b = b;
  a.y = y;
  if constexpr (sizeof(T) == 8) a.K = K64;
  else a.K = modal_to_f32(K64);
  a.sigma = T(0);
  a.omega = T(0.6);
  a.xin = nullptr;
  a.c1 = a.c2 = T(0);
  if (mode == OP_CHEB2) {  // in place over the previous iterate, as in the V-cycle
    a.xin = y;
    a.c1 = T(0.5);
    a.c2 = T(0.3);
  }
  a.kchunk = op_pick_kchunk<T>(G);
  a.diag_quirk = 1;
  const long long nb = op_num_blocks<T>(G, a.kchunk);
  if (!c.ensure_partials((size_t)nb * 2 + 64)) return HEXA_ERR_NOMEM;
  a.red.partials = c.partials;
  a.red.ticket = c.ticket;
  a.red.dst = c.dscal + 40;
  a.red.s = nullptr;
  a.red.op = FIN_STORE;
  a.red.nsum = 1;
  a.halt = nullptr;
  launch_op<T>(mode, a, c.st);  // warm-up
  cudaEventRecord(c.ev[0], c.st);
  for (int r = 0; r < reps; ++r) launch_op<T>(mode, a, c.st);
  cudaEventRecord(c.ev[1], c.st);
  c.launches += reps + 1;
  if (cudaEventSynchronize(c.ev[1]) != cudaSuccess || !c.cuda_ok("time_operator")) return set_err(h, HEXA_ERR_CUDA, c.err);
  if (!staging_ok(h, "time_operator")) return HEXA_ERR_CUDA;
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]);
  *avg_ms = ms / reps;
  c.last_ms = ms;
  return HEXA_OK;
}

extern "C" {

int hexa_time_operator(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, int32_t precision, int32_t mode,
                       const void* factor, const void* x, const void* b, void* y, int32_t reps, double* avg_ms) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !factor || !x || !y || !avg_ms || reps < 1 || mode < 0 || mode > 5)
    return set_err(h, HEXA_ERR_ARG, "invalid arguments");
  h->c.err.clear();
  cudaSetDevice(h->c.device);
  if (precision == HEXA_PREC_FP32)
    return time_operator_t<float>(h, g, bc, nu, mode, (const float*)factor, (const float*)x, (const float*)b, (float*)y,
                                  reps, avg_ms);
  return time_operator_t<double>(h, g, bc, nu, mode, (const double*)factor, (const double*)x, (const double*)b,
                                 (double*)y, reps, avg_ms);
}

int hexa_operator_diagonal(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, double nu, const double* factor,
                           int32_t diag_quirk, double* diag_out) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !factor || !diag_out) return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  ModalK<double> K64;
  std::string e;
  if (!build_modal(g->dx, g->dy, g->dz, nu, &K64, &e)) return set_err(h, HEXA_ERR_ARG, e);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  Mask m;
  m.faces = bc ? bc->clamp_faces : 0u;
  m.node = bc ? node_mask(c, G, bc->fixed_dof) : nullptr;
  const double* fac = stage_in<double>(c, factor, G.nelem(), "ap_fac64");
  double* d = out_buf<double>(c, diag_out, G.ndof(), "ap_y64");
  if (!fac || !d) return HEXA_ERR_NOMEM;
  launch_diag<double>(G, m, fac, K64, diag_quirk, 0.0, d, nullptr, c.st);
  c.launches++;
  stage_out<double>(c, diag_out, d, G.ndof());
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("diagonal")) return set_err(h, HEXA_ERR_CUDA, c.err);
  return HEXA_OK;
}

static bool valid_params(const hexa_solve_params* p) {
  return p && p->tol > 0 && p->max_iter >= 1 && p->nu > -1.0 && p->nu < 0.5 && p->shift_factor >= 0 &&
         (p->precision == HEXA_PREC_FP64 || p->precision == HEXA_PREC_FP32 || p->precision == HEXA_PREC_MIXED) &&
         (p->precond == HEXA_PRECOND_JACOBI || p->precond == HEXA_PRECOND_MULTIGRID);
}

int hexa_solve(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, const double* factor, const double* f,
               const hexa_solve_params* p, const double* u_guess, double* u_out, hexa_solve_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !factor || !f || !u_out) return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  if (!valid_params(p)) return set_err(h, HEXA_ERR_ARG, "invalid solver parameters");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  hexa_solve_stats st;
  std::memset(&st, 0, sizeof(st));
  Problem P;
  if (!prepare_problem(h, g, bc, p->nu, factor, f, &P)) return set_err(h, HEXA_ERR_NOMEM, c.err.empty() ? "staging failed" : c.err);
  const double* u0 = u_guess ? stage_in<double>(c, u_guess, P.g.ndof(), "in_u0") : nullptr;
  double* ud = out_buf<double>(c, u_out, P.g.ndof(), "out_u");
  if (!ud || (u_guess && !u0)) return set_err(h, HEXA_ERR_NOMEM, c.err);
  int rc = solve_problem(c, P, *p, u0, ud, &st);
  stage_out<double>(c, u_out, ud, P.g.ndof());
  if (cudaStreamSynchronize(c.st) != cudaSuccess) {
    c.cuda_ok("solve");
    rc = HEXA_ERR_CUDA;
  }
  if (!staging_ok(h, "solve")) rc = HEXA_ERR_CUDA;
  st.status = rc;
  st.total_ms = wall_ms(t0);
  c.last_ms = st.setup_ms + st.solve_ms;
  if (stats) *stats = st;
  return rc;
}

}  // extern "C"

// Body of the two reference-signature entries: the reference's Float32
// arguments converted on the host, optionally with the void pruning of
// Solver.solve_system (MeshPruner.prune_system, src/Mesh/MeshPruner.jl:10-87)
// restated on the structured grid.  Pruning removes the elements with density
// <= prune_thr and the nodes no kept element touches, then renumbers; on the
// structured grid the same system is the full grid with those elements'
// factors set to zero and the removed nodes' DOFs fixed: K_ff, f_free, the
// diagonal and its maximum (hence sigma) are then exactly the pruned
// system's, and the solver's zeros at fixed DOFs are what
// reconstruct_full_solution (MeshPruner.jl:89-107) writes at removed nodes.
static int solve_reference_args(hexa_ctx* h, const hexa_grid* g, float E, const float* bc_indicator, const float* f,
                                const float* density, bool prune, float prune_thr, const hexa_solve_params* p,
                                const float* u_guess, double* u_out, double* relres_out, char* method_out,
                                int32_t method_cap, hexa_solve_stats* stats, int64_t* active_out) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !f || !density || !u_out || !bc_indicator) return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  const long long NX = g->nx + 1, NY = g->ny + 1;
  const long long nn = NX * NY * (g->nz + 1);
  const long long ne = (long long)g->nx * g->ny * g->nz;
  // host conversion of the reference's Float32 arguments
  std::vector<float> hd(ne), hf(3 * nn), hb(3 * nn);
  auto fetch = [&](const float* src, float* dst, size_t n) {
    if (is_device_ptr(src)) cudaMemcpy(dst, src, n * sizeof(float), cudaMemcpyDeviceToHost);
    else std::memcpy(dst, src, n * sizeof(float));
  };
  fetch(density, hd.data(), ne);
  fetch(f, hf.data(), 3 * nn);
  fetch(bc_indicator, hb.data(), 3 * nn);
  std::vector<uint8_t> elem_on, node_on;
  long long nactive = ne;
  if (prune) {
    elem_on.assign(ne, 0);
    node_on.assign(nn, 0);
    nactive = 0;
    for (long long e = 0; e < ne; ++e) {
      if (!(hd[e] > prune_thr)) continue;  // active_mask = density .> threshold (MeshPruner.jl:20)
      elem_on[e] = 1;
      ++nactive;
      const long long i = e % g->nx, j = (e / g->nx) % g->ny, k = e / ((long long)g->nx * g->ny);
      for (int c = 0; c < 8; ++c)
        node_on[(i + (c & 1)) + NX * ((j + ((c >> 1) & 1)) + NY * (k + (c >> 2)))] = 1;
    }
    if (nactive == 0) {
      char msg[160];
      std::snprintf(msg, sizeof(msg), "MeshPruner: No active elements found (Threshold: %g). System is empty.",
                    (double)prune_thr);
      return set_err(h, HEXA_ERR_ARG, msg);
    }
  }
  if (active_out) *active_out = nactive;
  std::vector<double> fac(ne), fd(3 * nn), ug;
  for (long long e = 0; e < ne; ++e)  // Vector{T}(E .* density), GPUSolver.jl:254; pruned elements removed
    fac[e] = (prune && !elem_on[e]) ? 0.0 : (double)(float)(E * hd[e]);
  for (long long i = 0; i < 3 * nn; ++i) fd[i] = (double)hf[i];
  std::vector<uint8_t> fixed(3 * nn);
  for (long long n = 0; n < nn; ++n)
    for (int d = 0; d < 3; ++d)  // column-major Matrix(nNodes,3); removed nodes are not in the system
      fixed[3 * n + d] = (hb[n + nn * d] > 0.0f || (prune && !node_on[n])) ? 1 : 0;
  if (u_guess) {
    std::vector<float> hu(3 * nn);
    fetch(u_guess, hu.data(), 3 * nn);
    ug.assign(hu.begin(), hu.end());
  }
  hexa_bc bc;
  bc.clamp_faces = 0;
  bc.fixed_dof = fixed.data();
  hexa_solve_stats st;
  std::memset(&st, 0, sizeof(st));
  int rc = hexa_solve(h, g, &bc, fac.data(), fd.data(), p, u_guess ? ug.data() : nullptr, u_out, &st);
  if (relres_out) *relres_out = st.relres;
  if (method_out && method_cap > 0) {
    const char* name = (rc == HEXA_ERR_CORRUPT_INPUT) ? "Failed_Corrupt_Input"
                       : (st.precond_used == HEXA_PRECOND_USED_MULTIGRID ? "GMG_GPU" : "Jacobi_GPU");
    std::strncpy(method_out, name, (size_t)method_cap - 1);
    method_out[method_cap - 1] = 0;
  }
  if (stats) *stats = st;
  return rc;
}

extern "C" {

int hexa_solve_system_gpu(hexa_ctx* h, const hexa_grid* g, float E, const float* bc_indicator, const float* f,
                          const float* density, const hexa_solve_params* p, const float* u_guess, double* u_out,
                          double* relres_out, char* method_out, int32_t method_cap, hexa_solve_stats* stats) {
  return solve_reference_args(h, g, E, bc_indicator, f, density, false, 0.0f, p, u_guess, u_out, relres_out,
                              method_out, method_cap, stats, nullptr);
}

int hexa_solve_system(hexa_ctx* h, const hexa_grid* g, float E, const float* bc_indicator, const float* f,
                      const float* density, float min_stiffness_threshold, int32_t prune_voids,
                      int32_t current_outer_iter, const hexa_solve_params* p, const float* u_prev, double* u_out,
                      double* relres_out, char* method_out, int32_t method_cap, hexa_solve_stats* stats,
                      int64_t* active_elements) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !density) return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  // Solver.jl:66-72: the GPU solver type prunes from outer iteration 3 on
  bool prune = prune_voids != 0 && current_outer_iter >= 3;
  // Solver.jl:85-90: threshold min_stiffness_threshold * 1.01f0, pruned only below 99 % active
  const float thr = min_stiffness_threshold * 1.01f;
  if (prune) {
    const long long ne = (long long)g->nx * g->ny * g->nz;
    std::vector<float> hd(ne);
    if (is_device_ptr(density)) cudaMemcpy(hd.data(), density, ne * sizeof(float), cudaMemcpyDeviceToHost);
    else std::memcpy(hd.data(), density, ne * sizeof(float));
    long long nact = 0;
    for (long long e = 0; e < ne; ++e) nact += hd[e] > thr ? 1 : 0;
    prune = (double)nact < (double)ne * 0.99;
  }
  return solve_reference_args(h, g, E, bc_indicator, f, density, prune, thr, p, u_prev, u_out, relres_out,
                              method_out, method_cap, stats, active_elements);
}

int hexa_solve_multi_rhs(hexa_ctx* h, const hexa_grid* g, const hexa_bc* bc, const double* factor, int32_t k,
                         const double* F, const hexa_solve_params* p, double* U, hexa_solve_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !factor || !F || !U || k < 1) return set_err(h, HEXA_ERR_ARG, "invalid arguments");
  if (!valid_params(p)) return set_err(h, HEXA_ERR_ARG, "invalid solver parameters");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const long long ndof = 3LL * (g->nx + 1) * (g->ny + 1) * (g->nz + 1);
  hexa_solve_stats st;
  std::memset(&st, 0, sizeof(st));
  Problem P;
  // prepare_problem stages the factor and the first column; all k columns are staged here
  if (!prepare_problem(h, g, bc, p->nu, factor, F, &P)) return set_err(h, HEXA_ERR_NOMEM, c.err.empty() ? "staging failed" : c.err);
  const double* Fr = stage_in<double>(c, F, ndof * k, "in_F_raw");
  double* Fd = c.vec<double>("in_F", ndof * k);
  double* Ud = out_buf<double>(c, U, ndof * k, "out_U");
  if (!Fr || !Fd || !Ud) return set_err(h, HEXA_ERR_NOMEM, c.err);
  for (int j = 0; j < k; ++j) {  // loads at fixed DOFs are dropped, as in hexa_solve
    launch_mask_copy<double, double>(P.g, P.m, Fd + j * ndof, Fr + j * ndof, c.st);
    c.launches++;
  }
  int rc = multi_rhs_problem(c, P, k, Fd, *p, Ud, &st);
  stage_out<double>(c, U, Ud, ndof * k);
  if (cudaStreamSynchronize(c.st) != cudaSuccess) {
    c.cuda_ok("multi-rhs solve");
    rc = HEXA_ERR_CUDA;
  }
  if (!staging_ok(h, "multi-rhs solve")) rc = HEXA_ERR_CUDA;
  st.status = rc;
  st.total_ms = wall_ms(t0);
  c.last_ms = st.setup_ms + st.solve_ms;
  if (stats) *stats = st;
  return rc;
}

}  // extern "C"

// The filter's PCG on a device density of type T (GPUHelmholtz.jl:180-260):
// writes the filtered element field into outT, or sets *zero and leaves outT
// alone when the right-hand side is zero (the reference returns its input
// unchanged, GPUHelmholtz.jl:203-206).
template <typename T>
static int filter_run(hexa_ctx* h, const Grid& G, const T* rho, const HelmK& K, double tol, int max_iter, T* outT,
                      hexa_filter_stats* st, bool* zero) {
  Ctx& c = h->c;
  const long long nn = G.nnode();
  const char* tg = sizeof(T) == 8 ? "h64_" : "h32_";
  auto nm = [&](const char* s) { return std::string(tg) + s; };
  T* b = c.vec<T>(nm("b"), nn);
  T* x = c.vec<T>(nm("x"), nn);
  T* r = c.vec<T>(nm("r"), nn);
  T* z = c.vec<T>(nm("z"), nn);
  T* p = c.vec<T>(nm("p"), nn);
  T* q = c.vec<T>(nm("q"), nn);
  T* dinv = c.vec<T>(nm("dinv"), nn);
  if (!b || !x || !r || !z || !p || !q || !dinv) return HEXA_ERR_NOMEM;
  *zero = false;
  launch_helm_rhs<T>(G, rho, (T)K.rhs_scale, b, c.st);
  launch_helm_dinv<T>(G, K, dinv, c.st);
  c.launches += 2;
  RedArgs rd;
  rd.partials = c.partials;
  rd.ticket = c.ticket;
  rd.s = c.s;
  rd.dst = c.dscal + 20;
  rd.op = FIN_STORE;
  rd.nsum = 1;
  launch_dot<T>(b, b, (const T*)nullptr, (const T*)nullptr, nn, rd, kRed, nullptr, c.st);
  c.launches++;
  cudaMemcpyAsync(c.hscal + 20, c.dscal + 20, sizeof(double), cudaMemcpyDeviceToHost, c.st);
  cudaStreamSynchronize(c.st);
  const double bnorm = std::sqrt(c.hscal[20]);
  if (bnorm == 0.0) {
    *zero = true;
    st->iterations = 0;
    st->relres = 0.0;
    st->solve_ms = 0.0;
    return HEXA_OK;
  }
  PcgScalars hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.tol = tol;
  hs.max_iter = max_iter;
  hs.cadence = -10;
  hs.no_div = 1;
  hs.bnorm = bnorm;
  hs.best_rel = INFINITY;
  *c.hs = hs;
  cudaMemcpyAsync(c.s, c.hs, sizeof(PcgScalars), cudaMemcpyHostToDevice, c.st);
  launch_fill<T>(x, T(0), nn, c.st);
  launch_copy<T>(r, b, nn, c.st);
  c.launches += 2;
  rd.s = c.s;
  rd.op = FIN_INIT_RZ;
  launch_jacobi_precond<T>(z, r, dinv, nn, rd, kRed, nullptr, c.st);
  launch_copy<T>(p, z, nn, c.st);
  c.launches += 2;
  cudaEventRecord(c.ev[0], c.st);
  const int* halt = &c.s->halt;
  const int hblocks = (int)std::min<long long>((nn + 255) / 256, 152 * 8);
  while (true) {
    for (int it = 0; it < 10; ++it) {
      RedArgs ra = rd;
      ra.op = FIN_PCG_ALPHA;
      launch_helm_apply_dot<T>(G, K, p, q, ra, hblocks, halt, c.st);
      RedArgs rb = rd;
      rb.op = FIN_PCG_RES;
      rb.nsum = 2;
      launch_pcg_update<T>(x, r, z, p, q, dinv, nn, rb, kRed, c.s, c.st);
      launch_p_update<T>(p, z, nn, c.s, c.st);
      c.launches += 3;
    }
    cudaMemcpyAsync(c.hs, c.s, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) return HEXA_ERR_CUDA;
    if (c.hs->halt) break;
  }
  if (c.hs->status == 2 || c.hs->status == 4) {
    // a NaN residual or a breakdown of p.Ap: the reference's loop goes on with
    // alpha = rho / p.Ap non-finite and returns a NaN field (its callers test
    // for that, TopOpt.jl:360-363), so the output is NaN here too
    launch_fill<T>(outT, std::numeric_limits<T>::quiet_NaN(), G.nelem(), c.st);
  } else {
    launch_helm_extract<T>(G, x, outT, c.st);
  }
  c.launches++;
  cudaEventRecord(c.ev[1], c.st);
  cudaEventSynchronize(c.ev[1]);
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]);
  st->solve_ms = ms;
  st->iterations = c.hs->iter;
  st->relres = c.hs->relres;
  return HEXA_OK;
}

template <typename T>
static int filter_t(hexa_ctx* h, const Grid& G, const double* rho_d, const HelmK& K, double tol, int max_iter,
                    double* out_d, hexa_filter_stats* st) {
  Ctx& c = h->c;
  const long long ne = G.nelem();
  const char* tg = sizeof(T) == 8 ? "h64_" : "h32_";
  T* rho = c.vec<T>(std::string(tg) + "rho", ne);
  T* outT = c.vec<T>(std::string(tg) + "out", ne);
  if (!rho || !outT) return HEXA_ERR_NOMEM;
  if constexpr (sizeof(T) == 8) cudaMemcpyAsync(rho, rho_d, ne * sizeof(double), cudaMemcpyDeviceToDevice, c.st);
  else {
    launch_convert<float, double>(rho, rho_d, ne, c.st);
    c.launches++;
  }
  bool zero = false;
  const int rc = filter_run<T>(h, G, rho, K, tol, max_iter, outT, st, &zero);
  if (rc != HEXA_OK) return rc;
  if (zero) {
    cudaMemcpyAsync(out_d, rho_d, ne * sizeof(double), cudaMemcpyDeviceToDevice, c.st);
  } else if constexpr (sizeof(T) == 8) {
    cudaMemcpyAsync(out_d, outT, ne * sizeof(double), cudaMemcpyDeviceToDevice, c.st);
  } else {
    launch_convert<double, float>(out_d, outT, ne, c.st);
    c.launches++;
  }
  return HEXA_OK;
}

extern "C" {

int hexa_filter(hexa_ctx* h, const hexa_grid* g, const double* rho_in, double radius, double tol, int32_t max_iter,
                int32_t quirk, int32_t precision, double* rho_out, hexa_filter_stats* stats) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !rho_in || !rho_out || !(radius >= 0) || !(tol > 0) || max_iter < 1)
    return set_err(h, HEXA_ERR_ARG, "invalid filter arguments");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  double Ke[64], Me[64];
  if (scalar_matrices(g->dx, g->dy, g->dz, quirk, Ke, Me) != 0) return set_err(h, HEXA_ERR_ARG, "invalid element size");
  HelmK K;
  helm_corner_matrix(Ke, Me, radius, K.A);
  K.rhs_scale = g->dx * g->dy * g->dz / 8.0;  // GPUHelmholtz.jl:198-199
  const double* rd = stage_in<double>(c, rho_in, G.nelem(), "f_in");
  double* od = out_buf<double>(c, rho_out, G.nelem(), "f_out");
  if (!rd || !od) return HEXA_ERR_NOMEM;
  hexa_filter_stats st;
  std::memset(&st, 0, sizeof(st));
  const int rc = (precision == HEXA_PREC_FP32) ? filter_t<float>(h, G, rd, K, tol, max_iter, od, &st)
                                               : filter_t<double>(h, G, rd, K, tol, max_iter, od, &st);
  stage_out<double>(c, rho_out, od, G.nelem());
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("filter")) return set_err(h, HEXA_ERR_CUDA, c.err);
  st.status = rc;
  c.last_ms = st.solve_ms;
  if (stats) *stats = st;
  return rc;
}

void hexa_default_density_update_params(hexa_density_update_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->E = 1.0f;
  p->l1_stress_allowable = 1.0f;
  p->iter = 1;
  p->number_of_iterations = 30;  // config number_of_iterations (Main.jl:316)
  p->min_density = 1.0e-3f;
  p->max_density = 1.0f;
  p->filter_R_interm_iter_perc = 50.0f;
  p->minimum_filter_radius_as_elements = 2.5f;
  p->filter_tolerance = 1.0e-5f;
  p->final_density_threshold = 0.95f;
  p->max_culling_ratio = 0.1f;
  p->hard_update = 0;
  p->filter_max_iter = 200;
  p->filter_precision = HEXA_PREC_FP32;
}

// The filter radius schedule of TopOpt.jl:265-298 in Float32: linear from
// the initial to the intermediate radius up to the intermediate iteration,
// then to the final radius, floored at minimum_filter_radius_as_elements
// times the mean element size.  Host code is built without FMA contraction,
// so each product and sum rounds once as in the reference.
static float density_filter_radius(const hexa_density_update_params& p, float dx, float dy, float dz) {
  const float interm_frac = p.filter_R_interm_iter_perc / 100.0f;
  const float r_init = p.filter_R_init_perc / 100.0f * p.max_domain_dim;
  const float r_interm = p.filter_R_interm_perc / 100.0f * p.max_domain_dim;
  const float r_final = p.filter_R_final_perc / 100.0f * p.max_domain_dim;
  const int n = p.number_of_iterations;
  const int interm = std::max(1, (int)std::nearbyint(interm_frac * (float)n));  // round(Int, .): ties to even
  const int calc = std::min(p.iter, n);
  float r;
  if (calc <= interm) {
    const float t = interm > 1 ? (float)(calc - 1) / (float)(interm - 1) : 0.0f;
    r = r_init * (1.0f - t) + r_interm * t;
  } else {
    const float t = n > interm ? (float)(calc - interm) / (float)(n - interm) : 0.0f;
    r = r_interm * (1.0f - t) + r_final * t;
  }
  const float safe = p.minimum_filter_radius_as_elements * ((dx + dy + dz) / 3.0f);
  return r < safe ? safe : r;
}

// The culling threshold of TopOpt.jl:420-428.
static float density_cull_threshold(const hexa_density_update_params& p) {
  if (p.iter > p.number_of_iterations) return p.final_density_threshold;
  float prog = (float)p.iter / (float)p.number_of_iterations;
  prog = prog > 1.0f ? 1.0f : (prog < 0.0f ? 0.0f : prog);
  return p.final_density_threshold * prog;
}

int hexa_update_density(hexa_ctx* h, const hexa_grid* g, float* density, const float* l1_stress,
                        const uint8_t* protected_mask, const float* original_density,
                        const hexa_density_update_params* p, hexa_density_update_stats* stats) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !density || !l1_stress || !original_density || !p)
    return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  if (p->number_of_iterations < 1 || !(p->E > 0.0f) || !(p->l1_stress_allowable > 0.0f) || !std::isfinite(p->E) ||
      !std::isfinite(p->l1_stress_allowable) || !(p->filter_tolerance > 0.0f) || p->filter_max_iter < 1 ||
      !(p->min_density <= p->max_density) || !std::isfinite(p->min_density) || !std::isfinite(p->max_density) ||
      !(p->max_culling_ratio >= 0.0f) || !std::isfinite(p->max_culling_ratio) ||
      !std::isfinite(p->final_density_threshold))
    return set_err(h, HEXA_ERR_ARG, "invalid density update parameters");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  const long long ne = G.nelem();
  if (ne >= (1LL << 32)) return set_err(h, HEXA_ERR_TOO_LARGE, "density update: more than 2^32 - 1 elements");
  hexa_density_update_stats st;
  std::memset(&st, 0, sizeof(st));
  const float* l1d = stage_in<float>(c, l1_stress, ne, "ud_l1");
  const float* od = stage_in<float>(c, original_density, ne, "ud_orig");
  const uint8_t* pd = protected_mask ? stage_in<uint8_t>(c, protected_mask, ne, "ud_prot") : nullptr;
  const float* dd = stage_in<float>(c, (const float*)density, ne, "ud_rho");  // the user's array is written last
  float* prop = c.vec<float>("ud_prop", ne);
  float* work = c.vec<float>("ud_new", ne);
  UpdateState* s = c.vec<UpdateState>("ud_state", 1);
  double* part = c.vec<double>("ud_part", update_partials_doubles());
  unsigned long long* hist = c.vec<unsigned long long>("ud_hist", update_hist_bins());
  if (!l1d || !od || (protected_mask && !pd) || !dd || !prop || !work || !s || !part || !hist)
    return set_err(h, HEXA_ERR_NOMEM, c.err.empty() ? "density update: out of device memory" : c.err);
  static_assert(sizeof(UpdateState) <= 16 * sizeof(double), "UpdateState exceeds its host landing slots");
  UpdateState* hs = reinterpret_cast<UpdateState*>(c.hscal + 48);
  auto fetch = [&]() {
    cudaMemcpyAsync(hs, s, sizeof(UpdateState), cudaMemcpyDeviceToHost, c.st);
    return cudaStreamSynchronize(c.st) == cudaSuccess && c.cuda_ok("update_density");
  };
  cudaMemsetAsync(s, 0, sizeof(UpdateState), c.st);
  launch_propose(ne, l1d, pd, od, p->l1_stress_allowable, p->E, p->min_density, prop, s, c.st);
  c.launches++;
  if (!fetch()) return set_err(h, HEXA_ERR_CUDA, c.err);
  if (hs->nan_stress) {  // TopOpt.jl:230-236: no update, zero statistics
    st.status = 1;
    if (stats) *stats = st;
    return HEXA_OK;
  }
  st.R_length = density_filter_radius(*p, (float)g->dx, (float)g->dy, (float)g->dz);
  st.R_effective = st.R_length / 2.5f;
  st.current_threshold = density_cull_threshold(*p);
  const float* src = prop;
  if ((double)st.R_effective > 1e-4) {
    st.filter_used = 1;
    double Ke[64], Me[64];
    if (scalar_matrices(g->dx, g->dy, g->dz, 1, Ke, Me) != 0) return set_err(h, HEXA_ERR_ARG, "invalid element size");
    HelmK K;
    helm_corner_matrix(Ke, Me, (double)st.R_effective, K.A);
    K.rhs_scale = g->dx * g->dy * g->dz / 8.0;  // GPUHelmholtz.jl:198-199
    hexa_filter_stats fs;
    std::memset(&fs, 0, sizeof(fs));
    bool zero = false;
    int rc;
    if (p->filter_precision == HEXA_PREC_FP64) {
      double* p64 = c.vec<double>("h64_rho", ne);
      double* o64 = c.vec<double>("h64_out", ne);
      float* filt = c.vec<float>("ud_filt", ne);
      if (!p64 || !o64 || !filt) return set_err(h, HEXA_ERR_NOMEM, "density update: out of device memory");
      launch_convert<double, float>(p64, prop, ne, c.st);
      c.launches++;
      rc = filter_run<double>(h, G, p64, K, p->filter_tolerance, p->filter_max_iter, o64, &fs, &zero);
      if (rc == HEXA_OK && !zero) {
        launch_convert<float, double>(filt, o64, ne, c.st);
        c.launches++;
        src = filt;
      }
    } else {
      float* filt = c.vec<float>("h32_out", ne);
      if (!filt) return set_err(h, HEXA_ERR_NOMEM, "density update: out of device memory");
      rc = filter_run<float>(h, G, prop, K, p->filter_tolerance, p->filter_max_iter, filt, &fs, &zero);
      if (rc == HEXA_OK && !zero) src = filt;
    }
    if (rc != HEXA_OK) return set_err(h, rc, c.err.empty() ? "density update: filter failed" : c.err);
    st.filter_time = fs.solve_ms / 1e3;
    st.filter_iters = fs.iterations;
    st.filter_res = fs.relres;
  }
  c.launches += launch_update_cull(ne, dd, src, pd, od, p->min_density, p->max_density, st.current_threshold,
                                   p->max_culling_ratio, p->hard_update ? 1 : 0, work, part, hist, s, c.st);
  if (!fetch()) return set_err(h, HEXA_ERR_CUDA, c.err);
  if (hs->nan_filtered && src != prop) {  // TopOpt.jl:360-363: the unfiltered proposal instead
    st.filter_nan_fallback = 1;
    c.launches += launch_update_cull(ne, dd, prop, pd, od, p->min_density, p->max_density, st.current_threshold,
                                     p->max_culling_ratio, p->hard_update ? 1 : 0, work, part, hist, s, c.st);
    if (!fetch()) return set_err(h, HEXA_ERR_CUDA, c.err);
  }
  st.mean_change = hs->mean_change;
  st.active_count = (int64_t)hs->active;
  st.candidates = (int64_t)hs->candidates;
  st.culled = (int64_t)hs->culled;
  cudaMemcpyAsync(density, work, ne * sizeof(float),
                  is_device_ptr(density) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c.st);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("update_density")) return set_err(h, HEXA_ERR_CUDA, c.err);
  if (stats) *stats = st;
  return HEXA_OK;
}

int hexa_solve_batch(hexa_ctx* h, int32_t count, const hexa_grid* grids, const hexa_bc* bcs, double nu,
                     const double* const* factors, const double* const* forces, const hexa_solve_params* p,
                     double* const* u_out, hexa_solve_stats* stats) {
  if (!h) return HEXA_ERR_ARG;
  if (count < 1 || !grids || !factors || !forces || !u_out) return set_err(h, HEXA_ERR_ARG, "invalid batch arguments");
  if (!valid_params(p) || !(nu > -1.0 && nu < 0.5)) return set_err(h, HEXA_ERR_ARG, "invalid solver parameters");
  for (int i = 0; i < count; ++i)
    if (!valid_grid(grids + i) || !factors[i] || !forces[i] || !u_out[i])
      return set_err(h, HEXA_ERR_ARG, "invalid grid or null array in instance " + std::to_string(i));
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  int rc = batch_problem(c, count, grids, bcs, nu, factors, forces, *p, u_out, stats);
  if (rc < 0 && c.err.empty()) c.err = "batch solve failed";
  if (!staging_ok(h, "batch solve")) rc = HEXA_ERR_CUDA;
  return rc;
}

int hexa_filter_batch(hexa_ctx* h, int32_t count, const hexa_grid* grids, const double* const* rho_in, double radius,
                      double tol, int32_t max_iter, int32_t quirk, int32_t precision, double* const* rho_out,
                      hexa_filter_stats* stats) {
  if (!h) return HEXA_ERR_ARG;
  if (count < 1 || !grids || !rho_in || !rho_out || !(radius >= 0) || !(tol > 0) || max_iter < 1)
    return set_err(h, HEXA_ERR_ARG, "invalid batch filter arguments");
  for (int i = 0; i < count; ++i)
    if (!valid_grid(grids + i) || !rho_in[i] || !rho_out[i])
      return set_err(h, HEXA_ERR_ARG, "invalid grid or null array in instance " + std::to_string(i));
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = batch_filter(c, count, grids, rho_in, radius, tol, max_iter, quirk, precision, rho_out, stats);
  if (stats && rc == HEXA_OK) {
    const double ms = wall_ms(t0);
    for (int i = 0; i < count; ++i) stats[i].solve_ms = ms;
  }
  if (rc < 0 && c.err.empty()) c.err = "batch filter failed";
  return rc;
}

int hexa_stress_field(hexa_ctx* h, const hexa_grid* g, const double* u, const float* density, float E, float nu,
                      float* principal, float* vonmises, float* voigt, float* l1, float* dir_max, float* dir_min) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !u || !density || !principal || !vonmises || !l1 || !dir_max || !dir_min)
    return set_err(h, HEXA_ERR_ARG, "invalid grid or null array");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  const long long ne = G.nelem();
  const double* ud = stage_in<double>(c, u, G.ndof(), "st_u");
  const float* rd = stage_in<float>(c, density, ne, "st_rho");
  float* pd = out_buf<float>(c, principal, 3 * ne, "st_p");
  float* vd = out_buf<float>(c, vonmises, ne, "st_vm");
  float* wd = voigt ? out_buf<float>(c, voigt, 6 * ne, "st_w") : nullptr;
  float* ld = out_buf<float>(c, l1, ne, "st_l1");
  float* xd = out_buf<float>(c, dir_max, 3 * ne, "st_dmax");
  float* nd = out_buf<float>(c, dir_min, 3 * ne, "st_dmin");
  if (!ud || !rd || !pd || !vd || (voigt && !wd) || !ld || !xd || !nd) return set_err(h, HEXA_ERR_NOMEM, c.err);
  launch_stress<double>(G, ud, rd, E, nu, (float)g->dx, (float)g->dy, (float)g->dz, voigt ? 1 : 0, pd, vd, wd, ld, xd,
                        nd, c.st);
  c.launches++;
  stage_out<float>(c, principal, pd, 3 * ne);
  stage_out<float>(c, vonmises, vd, ne);
  if (voigt) stage_out<float>(c, voigt, wd, 6 * ne);
  stage_out<float>(c, l1, ld, ne);
  stage_out<float>(c, dir_max, xd, 3 * ne);
  stage_out<float>(c, dir_min, nd, 3 * ne);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("stress")) return set_err(h, HEXA_ERR_CUDA, c.err);
  return HEXA_OK;
}

int hexa_remap_fields(hexa_ctx* h, const hexa_grid* og, const hexa_grid* ng, double lx, double ly, double lz,
                      const float* density, const float* alpha, int32_t projection, float* new_density,
                      float* new_alpha) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(og) || !valid_grid(ng) || !density || !new_density || !(lx > 0 && ly > 0 && lz > 0))
    return set_err(h, HEXA_ERR_ARG, "invalid grids, lengths or null array");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const long long no = (long long)og->nx * og->ny * og->nz, nn = (long long)ng->nx * ng->ny * ng->nz;
  const float* dd = stage_in<float>(c, density, no, "rm_d");
  const float* ad = alpha ? stage_in<float>(c, alpha, no, "rm_a") : nullptr;
  float* ndd = out_buf<float>(c, new_density, nn, "rm_nd");
  float* nad = new_alpha ? out_buf<float>(c, new_alpha, nn, "rm_na") : nullptr;
  if (!dd || (alpha && !ad) || !ndd || (new_alpha && !nad)) return set_err(h, HEXA_ERR_NOMEM, c.err);
  launch_remap(og->nx, og->ny, og->nz, ng->nx, ng->ny, ng->nz, (float)ng->dx, (float)ng->dy, (float)ng->dz, (float)lx,
               (float)ly, (float)lz, projection ? 1 : 0, dd, ad, ndd, nad, c.st);
  c.launches++;
  stage_out<float>(c, new_density, ndd, nn);
  if (new_alpha) stage_out<float>(c, new_alpha, nad, nn);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("remap")) return set_err(h, HEXA_ERR_CUDA, c.err);
  return HEXA_OK;
}

int hexa_remap_displacement(hexa_ctx* h, const hexa_grid* og, const hexa_grid* ng, const double* u_old,
                            double* u_new) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(og) || !valid_grid(ng) || !u_old || !u_new) return set_err(h, HEXA_ERR_ARG, "invalid grids or null array");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const long long no = 3LL * (og->nx + 1) * (og->ny + 1) * (og->nz + 1);
  const long long nn = 3LL * (ng->nx + 1) * (ng->ny + 1) * (ng->nz + 1);
  const double* ud = stage_in<double>(c, u_old, no, "rm_u");
  double* und = out_buf<double>(c, u_new, nn, "rm_un");
  if (!ud || !und) return set_err(h, HEXA_ERR_NOMEM, c.err);
  launch_remap_nodal(og->nx, og->ny, og->nz, ng->nx, ng->ny, ng->nz, ud, und, c.st);
  c.launches++;
  stage_out<double>(c, u_new, und, nn);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("remap_displacement")) return set_err(h, HEXA_ERR_CUDA, c.err);
  return HEXA_OK;
}

int hexa_simp_factors(hexa_ctx* h, int64_t n, const double* rho, double Emin, double E0, double penal,
                      double* factor_out) {
  if (!h) return HEXA_ERR_ARG;
  if (n < 1 || !rho || !factor_out) return set_err(h, HEXA_ERR_ARG, "invalid arguments");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const double* rd = stage_in<double>(c, rho, n, "s_rho");
  double* fd = out_buf<double>(c, factor_out, n, "s_fac");
  if (!rd || !fd) return HEXA_ERR_NOMEM;
  launch_simp_factors(rd, Emin, E0, penal, fd, n, c.st);
  c.launches++;
  stage_out<double>(c, factor_out, fd, n);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("simp")) return set_err(h, HEXA_ERR_CUDA, c.err);
  return HEXA_OK;
}

int hexa_sensitivities(hexa_ctx* h, const hexa_grid* g, double nu, const double* rho, const double* u, double Emin,
                       double E0, double penal, double* dc_out, double* compliance_out) {
  if (!h) return HEXA_ERR_ARG;
  if (!valid_grid(g) || !rho || !u || !dc_out) return set_err(h, HEXA_ERR_ARG, "invalid arguments");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  ModalK<double> K64;
  std::string e;
  if (!build_modal(g->dx, g->dy, g->dz, nu, &K64, &e)) return set_err(h, HEXA_ERR_ARG, e);
  const Grid G = make_grid(g->nx, g->ny, g->nz);
  const double* rd = stage_in<double>(c, rho, G.nelem(), "s_rho");
  const double* ud = stage_in<double>(c, u, G.ndof(), "s_u");
  double* dd = out_buf<double>(c, dc_out, G.nelem(), "s_dc");
  if (!rd || !ud || !dd) return HEXA_ERR_NOMEM;
  RedArgs r;
  r.partials = c.partials;
  r.ticket = c.ticket;
  r.dst = c.dscal + 30;
  r.s = nullptr;
  r.op = FIN_STORE;
  r.nsum = 1;
  cudaEventRecord(c.ev[0], c.st);
  launch_sensitivities(G, K64, rd, ud, Emin, E0, penal, dd, r, c.st);
  cudaEventRecord(c.ev[1], c.st);
  c.launches++;
  cudaMemcpyAsync(c.hscal + 30, c.dscal + 30, sizeof(double), cudaMemcpyDeviceToHost, c.st);
  stage_out<double>(c, dc_out, dd, G.nelem());
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("sensitivities")) return set_err(h, HEXA_ERR_CUDA, c.err);
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]);
  c.last_ms = ms;
  if (compliance_out) *compliance_out = c.hscal[30];
  return HEXA_OK;
}

int hexa_oc_update(hexa_ctx* h, int64_t n, const double* x, const double* dc, const double* dv, double volfrac,
                   double move, double* x_out, double* lambda_out) {
  if (!h) return HEXA_ERR_ARG;
  if (n < 1 || !x || !dc || !dv || !x_out || !(volfrac > 0 && volfrac < 1) || !(move > 0))
    return set_err(h, HEXA_ERR_ARG, "invalid arguments");
  Ctx& c = h->c;
  c.err.clear();
  cudaSetDevice(c.device);
  const double* xd = stage_in<double>(c, x, n, "o_x");
  const double* cd = stage_in<double>(c, dc, n, "o_dc");
  const double* vd = stage_in<double>(c, dv, n, "o_dv");
  double* od = out_buf<double>(c, x_out, n, "o_out");
  double* lam_d = c.vec<double>("o_lam", 32);
  const int nb = (int)std::min<long long>((n + 255) / 256, 152 * 4);
  if (!xd || !cd || !vd || !od || !lam_d || !c.ensure_partials((size_t)nb * 32 + 64)) return HEXA_ERR_NOMEM;
  std::vector<double> part((size_t)nb * 32);
  // Bisection of the 88-line code on lambda in [0, 1e9] until
  // (l2-l1)/(l1+l2) <= 1e-3 is replaced by the same sequence of midpoints to a
  // tighter 1e-12, evaluated five levels of the bisection tree (31 multipliers)
  // per pass over the elements.
  double l1 = 0.0, l2 = 1e9, last_mid = 0.5 * (l1 + l2);
  const double target = volfrac * (double)n;
  int passes = 0;
  cudaEventRecord(c.ev[0], c.st);
  while ((l2 - l1) / (l1 + l2) > 1e-12 && passes < 64) {
    double lams[31];
    // heap order: node t has children 2t+1, 2t+2 (left = [l1,mid], right = [mid,l2])
    double lo[31], hi[31];
    lo[0] = l1;
    hi[0] = l2;
    for (int t = 0; t < 31; ++t) {
      lams[t] = 0.5 * (hi[t] + lo[t]);
      if (2 * t + 2 < 31) {
        lo[2 * t + 1] = lo[t];
        hi[2 * t + 1] = lams[t];
        lo[2 * t + 2] = lams[t];
        hi[2 * t + 2] = hi[t];
      }
    }
    cudaMemcpyAsync(lam_d, lams, sizeof(lams), cudaMemcpyHostToDevice, c.st);
    launch_oc_volumes(xd, cd, vd, n, lam_d, 31, move, c.partials, nb, c.st);
    c.launches++;
    cudaMemcpyAsync(part.data(), c.partials, (size_t)nb * 32 * sizeof(double), cudaMemcpyDeviceToHost, c.st);
    if (cudaStreamSynchronize(c.st) != cudaSuccess) return set_err(h, HEXA_ERR_CUDA, "oc pass failed");
    ++passes;
    int t = 0;
    for (int depth = 0; depth < 5; ++depth) {
      if (!((l2 - l1) / (l1 + l2) > 1e-12)) break;
      double vol = 0.0;
      for (int b = 0; b < nb; ++b) vol += part[(size_t)b * 32 + t];
      const double lmid = lams[t];
      last_mid = lmid;
      if (vol > target) {
        l1 = lmid;
        t = 2 * t + 2;
      } else {
        l2 = lmid;
        t = 2 * t + 1;
      }
    }
  }
  // the update is the one of the last midpoint tested, as in the 88-line loop
  const double lam = last_mid;
  launch_oc_apply(xd, cd, vd, n, lam, move, od, c.st);
  cudaEventRecord(c.ev[1], c.st);
  c.launches++;
  stage_out<double>(c, x_out, od, n);
  if (cudaStreamSynchronize(c.st) != cudaSuccess || !c.cuda_ok("oc")) return set_err(h, HEXA_ERR_CUDA, c.err);
  float ms = 0;
  cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]);
  c.last_ms = ms;
  if (lambda_out) *lambda_out = lam;
  return HEXA_OK;
}

}  // extern "C"
