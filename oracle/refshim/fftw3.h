/*
 * ORACLE build shim -- a project-written stand-in for the FFTW3 single-precision
 * API, declaring only what the reference's planning sources call
 * (dedispersion/msosm/msosm_prepare.cpp:179-221, overlap_save/osm_prepare.cpp:75-122).
 * FFTW itself is not installed.  The transforms are computed in double and
 * rounded to float (see fftw_shim.cpp), i.e. at least as accurate as fftwf.
 */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef float fftwf_complex[2];
typedef struct orc_fftwf_plan_s *fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_destroy_plan(fftwf_plan p);
#ifdef __cplusplus
}
#endif
