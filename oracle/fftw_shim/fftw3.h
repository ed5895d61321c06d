/*
 * fftw3.h -- minimal FFTW3-API shim used ONLY to compile the reference's own
 * sources into the test oracle (oracle/_ref).  FFTW3 is not installed on this
 * machine.  The transform is the plain DFT FFTW defines (FFTW_FORWARD =
 * exp(-2 pi i jk/n), unnormalized), computed in FP64 by ofc_dft() from
 * oracle/focss_oracle.c.  Only the calls the reference makes are provided
 * (src/focss/field.cpp:33,344,350,534-545, src/focss/functions.cpp:109-145).
 */
#ifndef FOCSS_FFTW_SHIM_H_
#define FOCSS_FFTW_SHIM_H_
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct fftw_plan_s* fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
fftw_complex* fftw_alloc_complex(size_t n);
void fftw_free(void* p);
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in,
                             const int* inembed, int istride, int idist, fftw_complex* out,
                             const int* onembed, int ostride, int odist, int sign,
                             unsigned flags);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#ifdef __cplusplus
}
#endif
#endif
