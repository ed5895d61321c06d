/* fftw_shim.c -- implementation of the FFTW3-API shim (see fftw3.h).  Test
 * infrastructure: linked only into oracle/_ref. */
#include "fftw3.h"
#include <stdlib.h>
#include <string.h>
#include "../focss_oracle.h"

struct fftw_plan_s {
    int n, howmany, istride, idist, ostride, odist, sign;
    fftw_complex *in, *out;
};

fftw_complex* fftw_alloc_complex(size_t n) {
    void* p = NULL;
    if (posix_memalign(&p, 64, (n ? n : 1) * sizeof(fftw_complex)) != 0) return NULL;
    return (fftw_complex*)p;
}

void fftw_free(void* p) { free(p); }

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in,
                             const int* inembed, int istride, int idist, fftw_complex* out,
                             const int* onembed, int ostride, int odist, int sign,
                             unsigned flags) {
    (void)inembed; (void)onembed; (void)flags;
    if (rank != 1) return NULL;
    struct fftw_plan_s* p = (struct fftw_plan_s*)calloc(1, sizeof(*p));
    p->n = n[0]; p->howmany = howmany; p->istride = istride; p->idist = idist;
    p->ostride = ostride; p->odist = odist; p->sign = sign; p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
    return fftw_plan_many_dft(1, &n, 1, in, NULL, 1, n, out, NULL, 1, n, sign, flags);
}

void fftw_execute(const fftw_plan p) {
    if (!p) return;
    double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)(p->n ? p->n : 1));
    for (int h = 0; h < p->howmany; ++h) {
        for (int i = 0; i < p->n; ++i) {
            const double* s = p->in[(size_t)h * p->idist + (size_t)i * p->istride];
            buf[2 * i] = s[0];
            buf[2 * i + 1] = s[1];
        }
        ofc_dft(p->n, buf, p->sign);
        for (int i = 0; i < p->n; ++i) {
            double* d = p->out[(size_t)h * p->odist + (size_t)i * p->ostride];
            d[0] = buf[2 * i];
            d[1] = buf[2 * i + 1];
        }
    }
    free(buf);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
