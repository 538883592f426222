// engine.h - host-side internals of libswave shared by engine.cu and fwi.cu.
#pragma once

#include <map>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/swave.h"
#include "swave_dev.cuh"

struct DBuf {
  void *p = nullptr;
  size_t cap = 0;
};

#include "batch.cuh"

struct RunOpts {
  int chunk = 16;       // steps per captured graph
  bool use_graph = true;
  bool rigid = false;   // skip the Higdon boundary (exact-adjoint mode)
  swave::StepTile tile; // fused-step tile shape
  // Return once the phase is queued: the kernels record errors in the
  // context's "run_err" flag, which the caller zeroes before and reads after
  // its phases (no profiling, no host outputs).
  bool async_end = false;
};

struct sw_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::map<std::string, DBuf> bufs;
  std::vector<cudaEvent_t> ev;
  bool profiling = false;
  sw_stats stats{};
  RunOpts run_opts;
};

namespace swave {

using ::RunOpts;

struct InjPlan {
  int on = 0;
  int bi0 = 0, bi1 = 0, bj0 = 0, bj1 = 0, bk0 = 0, bk1 = 0;
  std::vector<int> off;
  std::vector<InjEntry> ent;
};

struct ExtPlan {
  int on = 0, mode = 0, nrec = 0;
  int mirror = 0;   // rec_type > 0: u(row) - u(-row)
  std::vector<int> ic;
  std::vector<float> wz, wx;
};

// Device-side arrays of one propagation (host coordinates are kept to build
// the injection / extraction plans).
struct DevIO {
  float *vel_pad = nullptr;
  const float *vel_phys_host = nullptr;
  int nsou = 0;
  const float *sou_coord = nullptr;
  const float *sou_trace_dev = nullptr;
  int nrec = 0;
  const float *rec_coord = nullptr;
  float *rec_trace_dev = nullptr;
  float *wave_dev = nullptr;
  float *image_dev = nullptr;
  float *image2_dev = nullptr;   // SW_IMG_AFWI_RHO: the density gradient
  float *illum_dev = nullptr;
  const float *ref_dev = nullptr;
  float *final_u2_host = nullptr;
  // Checkpointed phases: the phase starts from init_state instead of zero
  // fields and leaves its final state in save_state (device arrays of 4
  // padded fields: u_1, u0, u1, u2).  tcnt, when non-zero, is the first
  // time sample of the whole phase, which snapshot counting refers to.
  const float *init_state = nullptr;
  float *save_state = nullptr;
  int tcnt = 0;
  // Variable density: padded rho, delp = 1/rho2 (device) and the unpadded
  // rho on the host (injection weights v^2*rho).
  const float *rho_pad = nullptr;
  const float *delp = nullptr;
  const float *rho_phys_host = nullptr;
};

// A shot's model window (ModelSpace%oxw, nxw, ...).
struct Window {
  float oxw, oyw, endx, endy;
  int nxw, nyw;
};

// One shot of a propagation phase: its descriptor and device arrays.
struct PhaseShot {
  sw_prop_desc d;
  DevIO io;
};

int fail(sw_ctx *c, int code, const char *fmt, ...);

#define SW_STR2(x) #x
#define SW_STR(x) SW_STR2(x)
// Returns SW_CUDA_ERR from the enclosing function (which has `sw_ctx *c`)
// when a CUDA runtime call fails, naming the call site.
#define SW_CK(call)                                                              \
  do {                                                                           \
    cudaError_t sw_e_ = (call);                                                  \
    if (sw_e_ != cudaSuccess)                                                    \
      return ::swave::cuda_fail(c, sw_e_, #call " @ " __FILE__ ":" SW_STR(__LINE__)); \
  } while (0)
int cuda_fail(sw_ctx *c, cudaError_t e, const char *what);
// cuTensorMapEncodeTiled from the driver (null when it is missing).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
// Grow-only named device buffer of the context; a growth allocates
// bytes + slack.
void *dbuf(sw_ctx *c, const std::string &name, size_t bytes, int *st, size_t slack = 0);
int check_genpar(sw_ctx *c, const sw_genpar &g);
Geom make_geom(const sw_genpar &g);
Coefs make_coefs(const sw_genpar &g);
// FD_acoustic_rho_init_coefs (FDcoefs.f90:12-23), coefpower = 1.
Coefs make_rho_coefs(const sw_genpar &g);
// Pads rho on the device like the velocity and forms delp = 1/rho2 with the
// half-cell sinc interpolation of Interpolate.f90:44-130 (slots "<slot>" and
// "<slot>_delp" of the context arena).
int prepare_rho(sw_ctx *c, const sw_genpar &g, const float *rho_host, const char *slot,
                const float **rho_pad, const float **delp);
void mksinc(float *sinc, int lsinc, float shift);
void compute_taper(int nxw, int nyw, std::vector<float> &tx, std::vector<float> &ty);
int build_injection(sw_ctx *c, const sw_genpar &g, const Geom &G, int mode, int nsou,
                    const float *sou_coord, const float *vel_phys, InjPlan &plan,
                    const float *rho_phys = nullptr, bool mirror = false);
int build_extraction(sw_ctx *c, const sw_genpar &g, const Geom &G, int mode, int nrec,
                     const float *rec_coord, ExtPlan &plan, bool mirror = false);
int run_phases(sw_ctx *c, std::vector<PhaseShot> &shots, const RunOpts &opt);
int compute_window(sw_ctx *c, const sw_genpar &g, float apx, float apy, const float *sou,
                   int nrec, const float *rec, Window &w);
void window_host(const sw_genpar &g, const Window &w, const float *big, std::vector<float> &small);
int propagate_dev(sw_ctx *c, const sw_prop_desc &d, const DevIO &io);
int upload_velocity(sw_ctx *c, const sw_genpar &g, const float *vel, const char *slot,
                    float **vel_pad);
int upload(sw_ctx *c, const char *slot, const void *h, size_t bytes, void **d);
int download(sw_ctx *c, void *h, const void *d, size_t bytes);

}  // namespace swave
