/* Header-only stand-in for GSL's wavelet API, enough to compile the
 * reference's Fwd.cpp as a test oracle.  The wavelet-compressed sensitivity
 * path (method_id 2) is not exercised by the oracle; every entry point aborts
 * so that an accidental call cannot go unnoticed. */
#ifndef GRADA_GSL_WAVELET_STUB_H
#define GRADA_GSL_WAVELET_STUB_H
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
typedef struct { int kind; } gsl_wavelet_type;
typedef struct { const gsl_wavelet_type *type; size_t k; } gsl_wavelet;
typedef struct { size_t n; } gsl_wavelet_workspace;
static const gsl_wavelet_type grada_stub_daub = {4};
static const gsl_wavelet_type *gsl_wavelet_daubechies = &grada_stub_daub;
static inline void grada_gsl_stub_abort(const char *fn)
{
  fprintf(stderr, "GSL stub: %s is not available in the oracle build\n", fn);
  abort();
}
static inline gsl_wavelet *gsl_wavelet_alloc(const gsl_wavelet_type *, size_t)
{ grada_gsl_stub_abort("gsl_wavelet_alloc"); return NULL; }
static inline gsl_wavelet_workspace *gsl_wavelet_workspace_alloc(size_t)
{ grada_gsl_stub_abort("gsl_wavelet_workspace_alloc"); return NULL; }
static inline void gsl_wavelet_free(gsl_wavelet *) { grada_gsl_stub_abort("gsl_wavelet_free"); }
static inline void gsl_wavelet_workspace_free(gsl_wavelet_workspace *)
{ grada_gsl_stub_abort("gsl_wavelet_workspace_free"); }
static inline int gsl_wavelet_transform_forward(const gsl_wavelet *, double *, size_t, size_t,
                                                gsl_wavelet_workspace *)
{ grada_gsl_stub_abort("gsl_wavelet_transform_forward"); return -1; }
static inline int gsl_wavelet_transform_inverse(const gsl_wavelet *, double *, size_t, size_t,
                                                gsl_wavelet_workspace *)
{ grada_gsl_stub_abort("gsl_wavelet_transform_inverse"); return -1; }
#endif
