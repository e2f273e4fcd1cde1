// Internal declarations shared by the host API (g4gpu_api.cpp) and the CUDA
// kernels (step_*.cu). Not part of the ABI.
#pragma once

#include <cstddef>
#include <cstdint>

#include <string>

#include "g4gpu.h"

namespace g4 {

// physical constants of the reference (src/Main/GenMain.cpp:63-68)
constexpr double kVacimp = 376.73;
constexpr double kEev = 510998.95069;
constexpr double kCe = 4.8032045e-11;

// Per field, per integration step constants.
struct FieldStep {
  double rtmp;    // fc(h) / xks of this field (BeamSolver.cpp:28)
  double rharm;   // harmonic number as a double (BeamSolver.cpp:30)
  double fc;      // fc(h) (Undulator.cpp:141-167), used by the deposition
  double xks;     // field wavenumber 2 pi h / lambda0 (Field.cpp:65)
  double gridmax; // half width of the grid (Field::gridmax)
  double dgrid;   // grid spacing 2 gridmax / (ngrid - 1) (Field.cpp:46)
  double cstep;   // imaginary part of the ADI step factor i dz / (4 xks dgrid^2)
  double k2scale; // FFT propagator: dk^2 dz / (2 xks)
  int dep_on;     // deposition active: in undulator and odd harmonic (FieldSolverADI.cpp:20)
  int coef;       // index of the ADI coefficient set of this (field, delz)
  int first;      // ring start of the field when the step runs (filled at launch)
  int tw;         // warm-up length of the segmented FP32 tridiagonal solves, 0: not applicable
  double idgrid;  // 1 / dgrid: the FP64 push's cell lookup multiplies
  double gm_idg;  // gridmax / dgrid: the FP64 cell coordinate is fma(x, idgrid, gm_idg)
  // The FP64 push forms e^{i h theta} at its RK4 stages by rotating e^{i h theta0}: by
  // e^{i h D} for the step's nominal phase advance D (StepConst::dnom_half over half a
  // step, dnom_full over the step) and by a short series for the small remainder.
  // rot_half / rot_full: cos and sin of rharm * dnom_half / dnom_full.
  double rot_half[2], rot_full[2];
  // cos and sin of rharm * autophase: the step's phase offset applied to a cached phasor
  double rot_auto[2];
};

// Per integration step constants (Undulator accessors, Undulator.h:82-204).
struct StepConst {
  // transverse optics, TrackBeam::track (TrackBeam.cpp:17-64)
  double aw_t;        // aw inside an undulator, else 0
  double qx, qy;      // focusing strengths
  double xoff, yoff;  // focusing centres (already divided by qx, qy)
  double cxk, cyk;    // corrector kicks times gamma0
  int kindx, kindy;   // 0 drift, 1 focusing, 2 defocusing
  int corr;           // corrector active at the end of the step
  int nfld;
  // longitudinal push, BeamSolver::advance (BeamSolver.cpp:13-87)
  double aw;          // aw[istepz] as BeamSolver reads it
  double ax, ay, kx, ky, gradx, grady;  // faw / faw2 (Undulator.cpp:170-182)
  double autophase;
  double xks;         // fundamental wavenumber
  double xku;         // undulator wavenumber, or xks/(2 gamma0^2) in drifts
  double delz;
  double gammaref;
  double ztemp1;      // -2 / xks (BeamSolver.cpp:147), the same value the ODE computes
  // exact products of the step's constants the FP64 push would otherwise form per
  // particle: delz / 2, aw_t^2, aw^2 (each the same IEEE product on the host)
  double half_delz, aw_t2, aw2;
  // nominal phase advance over half a step and over the step: delz / 2 and delz times
  // dtheta/dz of a particle at gammaref on axis without field (BeamSolver.cpp:144-163)
  double dnom_half, dnom_full;
  // chicane of the step (g4gpu_set_chicanes): its transfer matrix, applied before the
  // first half step (TrackBeam::applyChicane, TrackBeam.cpp:131-244), elements
  // m00 m01 m10 m11 m22 m23 m32 m33, and the phase shift R56 2 pi / (lambda0 gamma0)
  // per unit of gamma - gamma0 after the integration (TrackBeam::applyR56, :260-277)
  int chic;
  double cm[8];
  double r56;
  // incoherent synchrotron radiation (g4gpu_set_incoherent): the lattice's ku and helical
  // flag of the step, and the step's mean loss and spread half-width of gamma (0 off),
  // Incoherent::apply (Incoherent.cpp:31-63)
  double ku_raw;
  int helical;
  double isr_avg, isr_sig;
  FieldStep f[G4GPU_MAX_FIELDS];
};

// FP32 copy of the per-step constants for the mixed-precision kernels, prepared on
// the host so that no kernel converts FP64 constants per particle.
struct FieldStepF {
  float rtmp, rharm, gridmax, dgrid, cstep;
  float dep_scl;  // fc vacimp xks delz / (4 eev npart dgrid^2): times the slice current
  int dep_on, coef, first, harm;
  int tw;  // FieldStep::tw
};
struct StepConstF {
  float aw_t, qx, qy, xoff, yoff, cxk, cyk;
  int kindx, kindy, corr, nfld;
  float aw, ax, ay, kx, ky, gradx, grady;
  float xks, xku, delz, ztemp1;
  double autophase;
  long long autophase_q;  // autophase as a Q32.32 turn count
  double gammaref;
  int chic;  // StepConst::chic, cm, r56
  float cm[8];
  float r56;
  float isr_avg, isr_sig;  // StepConst::isr_avg, isr_sig
  FieldStepF f[G4GPU_MAX_FIELDS];
};
StepConstF to_float(const StepConst &s, int npart);

// Device arrays of one time window.
struct DeviceBeam {
  void *gamma, *theta, *x, *y, *px, *py;  // theta: FP64 (plain) or Q32.32 int64 (mixed), 8 B
  double *current;
  // particles of every slice when they differ (one4one windows: npart is then the
  // capacity of a slice), null when every slice holds npart
  int *count;
  // FP64 form: e^{i rharm theta} of every field and particle as the last push left it
  // ([nfield][nslice * npart] double2), and a device flag, nonzero while it matches theta
  // (cleared wherever theta is written outside the push); null in the mixed form
  void *phasor = nullptr;
  int *phasor_ok = nullptr;
};

struct Launch {
  void *stream;
  int *err;  // device error flag
};

// kernels_plain.cu (FP64, the reference's arithmetic)
// block: threads per block of the push (128, 256 or 512)
void launch_push_plain(const Launch &L, const StepConst &sc, const DeviceBeam &b,
                       void *const *field, void *const *src, int ns, int np, int ngrid,
                       int deposit, int block);
void launch_deposit_plain(const Launch &L, const StepConst &sc, const DeviceBeam &b,
                          void *const *src, int ns, int np, int ngrid);
// phase 0: implicit along x into tmp; phase 1: implicit along y back into the field
void launch_adi_plain(const Launch &L, const StepConst &sc, int k, int phase, void *field,
                      const void *src, void *tmp, const void *coef, int ns, int ngrid);
void launch_diag_beam_plain(const Launch &L, const DeviceBeam &b, int ns, int np, int nharm,
                            double *out);
void launch_diag_field_plain(const Launch &L, const void *field, int ns, int ngrid,
                             double *out);

// kernels_mixed.cu (FP32 field, FP64 phase)
void launch_push_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b,
                       void *const *field, void *const *src, int ns, int np, int ngrid,
                       int deposit, int block);
void launch_deposit_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b,
                          void *const *src, int ns, int np, int ngrid);
void launch_adi_mixed(const Launch &L, const StepConstF &sc, int k, int phase, void *field,
                      const void *src, void *tmp, const void *coef, int ns, int ngrid);
void launch_diag_beam_mixed(const Launch &L, const DeviceBeam &b, double gammaref, int ns, int np,
                            int nharm, double *out);
void launch_diag_field_mixed(const Launch &L, const void *field, int ns, int ngrid,
                             double *out);
// Fused deposition + ADI of one field in shared memory, one CTA per slice; usable
// for ngrid <= fused_max_ngrid() (168: the FP32 slice must fit in 227 KB).
int fused_max_ngrid();
// The same step on a thread-block cluster of cl CTAs per slice (2 <= cl <=
// kMaxBandCluster), each holding a band of the rows; usable when the step's segmented
// solves apply (FieldStep::tw > 0). band_cluster(ngrid, W) gives the smallest cluster
// whose bands fit shared memory with the last band at least W rows (the segments'
// warm-up), or 0 if none does.
constexpr int kMaxBandCluster = 4;
int band_cluster(int ngrid, int W);
void launch_field_band_mixed(const Launch &L, const StepConstF &sc, int k, const DeviceBeam &b, void *field,
                             const void *coef, int ns, int np, int ngrid, int deposit, int cl);
// threads: CTA size, a multiple of 32 in [2 ngrid, 1024]. dbeam / dfield (may be
// null): the step's diagnostic record, beam [nslice][beam_diag_width(nharm)] (formed by
// the launch of field 0) and this field's [nslice][kFieldSums + 2] in storage order.
void launch_field_fused_mixed(const Launch &L, const StepConstF &sc, int k, const DeviceBeam &b,
                              void *field, const void *coef, int ns, int np, int ngrid, int deposit,
                              int threads, double *dbeam, double *dfield, int nharm, double gref);
// One source sub-step of a coarse step (g4gpu_set_field_substeps; k_source_f): the
// deposition of every beam slice into field 0's slot (is + sc.f[0].first) % ns, u +=
// scale * src, from phases and positions interpolated at frac between tp, xp, yp (the
// beam before the push) and the beam's arrays. npart % 4 == 0, full slices.
void launch_source_substep_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b, const void *tp,
                                 const void *xp, const void *yp, float frac, float scale, void *field, int ns,
                                 int np, int ngrid);
// whether the fused kernel can record the diagnostics (nharm bunching harmonics) too
bool fused_diag_fits(int ngrid, int threads, int nharm);
// One ADI step of ns float2 field slices with an optional source, all scratch in the
// module's static device array (g4gpu_adi_advance_noalloc); coef: [3][ngrid] float2 of
// c, cbet, cwet. Synchronises `stream`. Returns a G4GPU_ERR_* code with *msg set.
size_t noalloc_scratch_bytes();
int adi_noalloc_mixed(int device, void *stream, void *field, const void *source, const float *coef,
                      float cstep, int ns, int ngrid, int first, std::string *msg);

// Incoherent synchrotron radiation: the random stream of the push. ctr: the device
// counter of steps drawn (advanced by launch_isr_advance after each push that draws),
// seed: &sponrad seed, nbins: particles that share a draw (a beamlet)
struct IsrStream {
  const unsigned long long *ctr;
  unsigned seed;
  int nbins;
};
void launch_isr_advance(void *stream, unsigned long long *ctr);

// The whole step of a one-field window in one kernel, one CTA per slice: push,
// deposition and ADI (mixed form, slice in shared memory, no space charge). Usable
// where step_fused_ok; threads, dbeam, dfield as launch_field_fused_mixed's; wake and
// isr as the push's.
bool step_fused_ok(int nfield, int ngrid, int threads, bool dbeam, bool dfield, int nharm);
void launch_step_fused_mixed(const Launch &L, const StepConstF &sc, const DeviceBeam &b, void *field,
                             const void *coef, int ns, int np, int ngrid, int deposit, int threads,
                             const void *wake, const IsrStream &isr, double *dbeam, double *dfield, int nharm,
                             double gref);

// Space charge (&efield, EFieldSolver.cpp), sc_kernels.cuh, instantiated in
// kernels_plain.cu (FP64) and kernels_mixed.cu (FP32).
struct ScConst {
  int ns, np, ng, nz, nphi;
  int longrange, shortrange;  // which parts run (EFieldSolver::hasShortRange: nz > 0, ngrid > 2)
  int modes_per_pass;         // radial modes the short-range kernel holds in shared memory at once
  double slicelength;         // lambda0 * sample
  double gamma_lr;            // gammaref / sqrt(1 + aw^2) of the step (EFieldSolver.cpp:69)
  double lr_scl;              // slicelength / (2 asin 1) / c / 2 / eps0 (EFieldSolver.cpp:103)
  double ks;                  // 2 pi / lambda0
  double coef;                // -gammaz^2 / ks^2 of the Laplace operator (EFieldSolver.cpp:217)
};
// device state of a handle's space charge
struct ScBuffers {
  double *st;       // [7][nslice]: xcen, ycen, size, rbound, rmax of the slice, eloss; 2 x nslice floats
  double *state;    // [1]: the radial grid extent carried over steps
  unsigned *count;  // CTAs of the moment kernel that finished (reset by the last)
  void *ez;         // [nslice][npart] R: short-range field per particle
};
// shared memory of the short-range kernel per mode, and the largest it takes
size_t sc_bytes_per_mode(int ng, int mixed);
size_t sc_max_smem();
// part 0: the first transverse half step of the push with the slice moments and the
// radial grid extents; part 1: the long-range loss and the short-range field. The push
// follows with mode 2.
void launch_sc_plain(const Launch &L, const ScConst &c, const StepConst &step, const DeviceBeam &b,
                     const ScBuffers &buf, int part);
void launch_sc_mixed(const Launch &L, const ScConst &c, const StepConstF &step, const DeviceBeam &b,
                     const ScBuffers &buf, int part);
// The push in parts: mode 1 the first transverse half step only; mode 2 the rest of the
// step with ez [nslice][npart] (may be null) plus eloss [nslice] (may be null) in the
// energy equation. Mode 0 is the whole step. wake [nslice] (may be null): the slices'
// wake loss added to gamma after the integration, eV/m as FP64 (plain) or divided by
// eev as FP32 (mixed).
void launch_push_plain_sc(const Launch &L, const StepConst &sc, const DeviceBeam &b, void *const *field,
                          void *const *src, int ns, int np, int ngrid, int deposit, int block, int mode,
                          const void *ez, const double *eloss, const void *wake, const IsrStream &isr);
void launch_push_mixed_sc(const Launch &L, const StepConstF &sc, const DeviceBeam &b, void *const *field,
                          void *const *src, int ns, int np, int ngrid, int deposit, int block, int mode,
                          const void *ez, const double *eloss, const void *wake, const IsrStream &isr);
// Wakes (Collective::update): loss [nslice] = ext + the wake of each slice from the
// window's current cur [nslice]; lossf = loss / eev in FP32; scratch: 2 ns_hr doubles.
void launch_wake_update(const Launch &L, const double *cur, int nslice, int ns_hr, double ds, const double *ext,
                        const double *res, const double *geo, const double *rou, double *scratch, double *loss,
                        float *lossf);

// kernels_sort.cu: one4one sorting (Beam::sort for one rank); b.count must be set.
// scratch: the six particle arrays' layout; iscratch: 3 ns + 1 ints, the last the number
// of particles that found no room in their slice
void launch_sort(void *stream, int mixed, const DeviceBeam &b, void *const *scratch, int *iscratch, int ns, int cap,
                 double lambda0, double sample);

// kernels_fft.cu: FFT field solver (FieldSolverFFT::FFT)
struct FFTPlan {
  int n, nstage;
  int radix[32];   // radices of the stages, whose product is n
  int tw_off[32];  // offset of each stage's twiddles in the table after the n roots
  int nb[32];      // n / radix
  // ceil(2^32 / d) for d = nb and d = ns (the product of the earlier radices): the
  // kernels divide small integers x (x d < 2^32) by them as one multiply-high
  unsigned mnb[32], mns[32];
  unsigned mn;  // ceil(2^32 / n)
};
int fft_max_ngrid(int mixed);
// lines of a slice one CTA transforms at a time in a pass with `bufs` tile buffers
// and `per_sm` CTAs on an SM (es: bytes of a complex element; at most maxL)
int fft_lines_per_cta(const FFTPlan &pl, int es, int bufs, int maxL, int per_sm);
// whether the kernels can take the plan's stages (one butterfly per thread for a
// line of each register stage, at most 8 outputs per thread of a generic one)
int fft_plan_fits(const FFTPlan &pl);
// roots: n complex exp(-2 pi i m / n) followed by the stage twiddles, stage s's
// exp(-2 pi i q k / (ns R)) at tw_off[s] + (q - 1) ns + k (ns the product of the
// earlier radices, R the stage's, 0 < q < R, k < ns), n - 1 in all; k2c:
// -dk^2 / (2 xks), Im(K2) = (dx^2 + dy^2) k2c; sig: the sigmoid filter on the FFT
// index (real, n^2, transposed: element kx n + ky); work: n^2 * nslice complex
// scratch, used when filtered
// Far-field moments of the field diagnostics: the row pass into `work` (n^2 nslice
// complex scratch), then the column pass that writes one partial of 5 sums per tile of
// fft_diag_lines columns: part[(ii nblk + blk) 5 + k], nblk = ceil(n / lines).
int fft_diag_lines(const FFTPlan &pl, int mixed);
void launch_fft_diag(void *stream, int mixed, const void *field, void *work, const void *roots, const FFTPlan &pl,
                     int ns, int first, double *part);
void launch_fft_solve(void *stream, int mixed, void *field, const void *src, void *work, const void *roots,
                      double k2c, const void *sig, int filtered, double delz, const FFTPlan &pl, int ns,
                      int first);

// kernels_mlp.cu: BF16 tensor-core MLP (tcgen05 fed by TMA, FP32 accumulation in
// tensor memory). mlp_gemm_nt needs N and K multiples of 16 (mlp_tile_n gives the
// tile width, 0 if unsupported) and returns -1 otherwise, -2 if the driver gives no
// tensor map for an operand (16-byte aligned operands only); *err (device) is set
// if a bounded wait for the copies or MMAs runs out. mlp_transpose_bf16 writes ldo >= rows
// columns, zero past rows.
int mlp_tile_n(int N, int K);
int mlp_gemm_nt(void *stream, const void *A, const void *B, const float *bias, float *C, void *Cb, int M, int N,
                int K, int relu, int accumulate, int *err);
void mlp_transpose_bf16(void *stream, const void *in, void *out, int rows, int cols, int ldo);
void mlp_to_bf16(void *stream, const float *in, void *out, size_t n);
void mlp_relu_backward(void *stream, const float *dA, const float *Z, float *dZ, void *dZb, size_t n);
void mlp_colsum(void *stream, const float *dZ, float *db, int rows, int cols);
void mlp_mse(void *stream, const float *Y, const float *T, float *dY, void *dYb, int rows, int nout, int ldy,
             float *loss);
void mlp_adam(void *stream, float *w, const float *g, float *m, float *v, size_t n, float lr, float b1,
              float b2, float eps, int t);

// kernels_closure.cu: per-slice features and corrections of the learned closure
constexpr int kClosureNin = 32;
constexpr int kClosureNout = 4;
void closure_features(void *stream, const void *theta, const void *gam, const double *current,
                      const void *field, const float *basis, int mixed, double gref, int ns, int np, int ng,
                      int first, float u0, float c0, float *out);
void closure_apply(void *stream, void *theta, void *gam, void *field, const float *corr, int mixed, int ns,
                   int np, int ng, int first);
void closure_targets(void *stream, const void *th_c, const void *g_c, const void *f_c, const void *th_f,
                     const void *g_f, const void *f_f, int mixed, int ns, int np, int ng, int first_c,
                     int first_f, float *out);
void closure_normalize(void *stream, const float *x, const float *mean, const float *stdv, void *yb, int rows,
                       int n, int ld);
void closure_denormalize(void *stream, const float *y, const float *scale, const float *shift, float *out,
                         int rows, int n, int ld);

// number of raw sums per slice written by the diagnostic kernels
constexpr int kBeamSums = 12;   // g1 g2 x1 x2 y1 y2 px1 px2 py1 py2 xpx ypy
constexpr int kBeamMinMax = 10; // xmin xmax pxmin pxmax ymin ymax pymin pymax gmin gmax
#ifdef __CUDACC__
__host__ __device__
#endif
inline int beam_diag_width(int nharm) { return kBeamSums + kBeamMinMax + 2 * nharm; }
constexpr int kFieldSums = 7;   // power x1 x2 y1 y2 ff.re ff.im

// host_loading.cpp
double host_fc(double aw, int helical, int h);

}  // namespace g4
