// The handle structure behind g4gpu_handle, shared by the host translation units
// (g4gpu_api.cpp, g4gpu_learned.cpp). Not part of the ABI.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "g4gpu.h"
#include "g4gpu_internal.h"

struct g4gpu_mlp_ctx;

struct g4gpu_ctx {
  g4gpu_config cfg{};
  cudaStream_t stream = nullptr;
  std::string err;
  bool mixed = false;
  size_t csize = 16;  // bytes per complex field value
  size_t rsize = 8;   // bytes per particle coordinate other than theta

  g4::DeviceBeam beam{};
  void *field[G4GPU_MAX_FIELDS] = {};
  void *src[G4GPU_MAX_FIELDS] = {};
  void *tmp = nullptr;
  void *diag_work = nullptr;  // g4gpu_diag_fft's scratch where tmp is absent
  void *coef = nullptr;      // [nset][3][ngrid] complex of the field type
  size_t coef_bytes = 0;
  // FFT solver tables per field: roots of unity [n], Im(K2) and the sigmoid [n^2]
  void *fft_roots[G4GPU_MAX_FIELDS] = {};
  double fft_k2c[G4GPU_MAX_FIELDS] = {};  // -dk^2 / (2 xks): Im(K2) = (dx^2 + dy^2) k2c
  void *fft_sig[G4GPU_MAX_FIELDS] = {};
  g4::FFTPlan fft_plan{};
  int *derr = nullptr;
  double *ddiag = nullptr;
  size_t ddiag_bytes = 0;
  double *hdiag = nullptr;  // pinned host copy of ddiag (the per-step read-back)
  // g4gpu_run_diag: the record of the step being queued (null otherwise), its
  // harmonics, and whether the step's kernels formed the fields' (and the beam's) part
  // of it
  double *diag_rec = nullptr;
  int diag_nharm = 0;
  bool diag_fields_in_step = false;
  bool diag_beam_in_step = false;
  // space charge (g4gpu_set_efield): its parameters and device state
  bool sc_on = false;
  int sc_ngrid = 0, sc_nz = 0, sc_nphi = 0, sc_longrange = 0;
  g4::ScBuffers sc{};
  // wakes (g4gpu_set_wake): fine-grid single-particle wakes, external loss, the slices'
  // loss (FP64 eV/m and FP32 over eev) and the update's scratch, all on the device
  bool wake_on = false;
  int wake_ns = 0;
  double wake_ds = 0, wake_ztrans = 0, wake_radius = 0;
  int wake_transient = 0;
  double *wake_tab = nullptr;  // [3][wake_ns] res, geo, rou (first points halved), then [nslice] ext
  double *wake_loss = nullptr;  // [nslice]
  float *wake_lossf = nullptr;  // [nslice]
  double *wake_scratch = nullptr;  // [2][wake_ns]
  // incoherent synchrotron radiation (g4gpu_set_incoherent): flags, seed, beamlet size and
  // the device counter of the steps that drew random numbers
  bool isr_loss = false, isr_spread = false;
  unsigned isr_seed = 0;
  int isr_nbins = 1;
  unsigned long long *isr_ctr = nullptr;
  // one4one windows (g4gpu_load_beam_counts): particles per slice on the device
  // (beam.count points at it then) and their host copy; the sort's scratch
  int *count_buf = nullptr;
  std::vector<int> hcount;
  void *sort_scratch[6] = {};
  int *sort_iscratch = nullptr;
  void *stage = nullptr;     // AoS staging buffer for host transfers
  size_t stage_bytes = 0;
  size_t bytes = 0;

  int nsteps = 0;
  std::vector<g4::StepConst> steps;
  std::vector<double> slip;
  // g4gpu_set_field_substeps: periods per lattice step (empty: none), and the beam's
  // phases and positions at the start of a coarse push
  std::vector<int> substeps;
  void *sub_theta = nullptr, *sub_x = nullptr, *sub_y = nullptr;
  int first[G4GPU_MAX_FIELDS] = {};
  double accuslip[G4GPU_MAX_FIELDS] = {};
  // sharded windows: the storage slot g4gpu_shift_out freed for the entering slice
  // (-1: none pending)
  int shift_slot[G4GPU_MAX_FIELDS] = {-1, -1, -1, -1, -1, -1, -1, -1};
  bool beam_loaded = false;
  bool field_loaded[G4GPU_MAX_FIELDS] = {};

  // launch shapes (chosen by g4gpu_autotune, defaults otherwise)
  int push_block = 256;
  int field_threads = 512;
  // mixed ADI with the slice in shared memory: 0 one CTA per slice (k_field_fused_f),
  // 1 a cluster pair (k_field_band_f<2>), 2 the whole step per CTA (k_step_fused_f)
  int field_kernel = 0;

  // captured step sequences, keyed by the step range and the ring state they start from
  bool graph_mode = false;
  struct GraphKey {
    int istep0, nsteps, stages, push_block, field_threads, field_kernel;
    std::vector<long long> state;  // first[] and the bit patterns of accuslip[]
    bool operator<(const GraphKey &o) const {
      return std::tie(istep0, nsteps, stages, push_block, field_threads, field_kernel, state) <
             std::tie(o.istep0, o.nsteps, o.stages, o.push_block, o.field_threads, o.field_kernel, o.state);
    }
  };
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::vector<int> end_first;
    std::vector<double> end_accuslip;
    long long launches[G4GPU_K_NCLASS] = {};
  };
  std::map<GraphKey, GraphEntry> graphs;
  // advanced whenever the captured graphs are dropped (a new lattice, chicanes, beam
  // layout, set-up), so that a batch's ensemble graphs of this member are not reused
  long long graph_gen = 0;
  bool capturing = false;

  // learned closure (g4gpu_learned.cpp)
  g4gpu_mlp_ctx *mlp = nullptr;
  float *closure_basis = nullptr;  // [4][ngrid] 1-D factors of the Gauss-Hermite modes of field 0
  float *closure_feat = nullptr;   // [nslice][32]
  float *closure_corr = nullptr;   // [nslice][4]
  float closure_u0 = 1.f, closure_c0 = 1.f;

  bool prof = false;
  long long launches[G4GPU_K_NCLASS] = {};
  double ms[G4GPU_K_NCLASS] = {};
  struct Pending {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
};

// shared helpers of the host translation units (g4gpu_api.cpp)
int g4_fail(g4gpu_handle h, int code, const std::string &msg);
int g4_cuda_fail(g4gpu_handle h, cudaError_t e, const char *what);
int g4_alloc(g4gpu_handle h, void **p, size_t n);
int g4_check_device_flag(g4gpu_handle h);
