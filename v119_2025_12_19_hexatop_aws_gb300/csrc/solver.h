// Library context and solver entry points (C++ side of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>

#include "../../include/hexagpu.h"
#include "hexa_common.cuh"

namespace hexa {

struct Ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::string err;
  double last_ms = 0.0;
  int64_t launches = 0;
  // growable named device buffers, reused across calls (the reference keeps
  // its workspaces in module globals, GPUSolver.jl:63)
  std::map<std::string, std::pair<void*, size_t>> bufs;
  double* partials = nullptr;
  size_t partials_cap = 0;  // doubles
  unsigned* ticket = nullptr;
  PcgScalars* s = nullptr;   // main PCG
  PcgScalars* s2 = nullptr;  // coarse-level PCG
  double* dscal = nullptr;   // 64 device doubles of scratch results
  PcgScalars* hs = nullptr;  // pinned host mirror of s
  // autotuned settings per problem: multigrid {levels, smoothing steps,
  // Chebyshev ratio}; batches {z-brick depth, -, -}
  struct Tuned {
    int a = 0, b = 0, c = 0;
  };
  std::map<std::string, Tuned> tuned;
  double* hscal = nullptr;   // pinned host mirror of dscal

  void* get(const std::string& name, size_t bytes);
  template <typename T>
  T* vec(const std::string& name, size_t n) { return (T*)get(name, n * sizeof(T)); }
  bool ensure_partials(size_t n);
  bool fail(const std::string& msg) { err = msg; return false; }
  bool cuda_ok(const char* where);
};

// Is p a device (or managed) pointer on this context's device?
bool is_device_ptr(const void* p);

struct Problem {
  Grid g;
  Mask m;                 // faces + device node mask (nullable)
  const double* fac64;    // device, nelem
  const double* f64;      // device, ndof, zero at fixed DOFs
  double dx, dy, dz, nu;
};

int solve_problem(Ctx& c, const Problem& P, const hexa_solve_params& prm, const double* u0_dev,
                  double* u_dev, hexa_solve_stats* st);
int multi_rhs_problem(Ctx& c, const Problem& P, int k, const double* F_dev,
                      const hexa_solve_params& prm, double* U_dev, hexa_solve_stats* st);

int batch_problem(Ctx& c, int count, const hexa_grid* grids, const hexa_bc* bcs, double nu,
                  const double* const* factors, const double* const* forces, const hexa_solve_params& prm,
                  double* const* u_out, hexa_solve_stats* stats);
int batch_filter(Ctx& c, int count, const hexa_grid* grids, const double* const* rho_in, double radius, double tol,
                 int max_iter, int quirk, int precision, double* const* rho_out, hexa_filter_stats* stats);

bool build_modal(double dx, double dy, double dz, double nu, ModalK<double>* K, std::string* err);

}  // namespace hexa
