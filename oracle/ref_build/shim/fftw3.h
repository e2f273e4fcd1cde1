/* Stand-in for the FFTW3 API (FFTW 3.3, www.fftw.org), used only to compile the
 * GENESIS 1.3 v4 reference sources with -DFFTW into a CPU checker (oracle/_ref), so
 * that the reference's own FFT field solver (src/Core/FieldSolverFFT.cpp:9-167) and
 * far-field diagnostics (src/Core/Diagnostic.cpp:614-847) run here, where FFTW is not
 * installed.
 *
 * The reference calls exactly five names of FFTW: fftw_complex, fftw_plan,
 * fftw_plan_dft_2d, fftw_execute and fftw_destroy_plan (src/Util/FFTObj.cpp:25-37,
 * src/Core/FieldSolverFFT.cpp:70-151, src/Core/Field.cpp:10-62,
 * src/Core/Diagnostic.cpp:749-790). This header declares them with FFTW's public
 * signatures and constants. What a plan computes is FFTW's documented transform, the
 * unnormalised 2-D DFT
 *     out[k0][k1] = sum_{j0,j1} in[j0][j1] exp(sign 2 pi i (j0 k0 / n0 + j1 k1 / n1)),
 * sign = FFTW_FORWARD (-1) or FFTW_BACKWARD (+1), row-major arrays. The implementation
 * (g4ref_fftw.cpp) evaluates that sum directly in extended precision; it is test
 * infrastructure written for this project and contains no FFTW code. */
#ifndef G4REF_FFTW3_SHIM_H
#define G4REF_FFTW3_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
