/* wl_host.h -- ensemble files of the C host layer (libwlhost.so).
 *
 * No counterpart in the reference, which reads loops only from its text
 * format (getwl, declared in wl_legacy.h, getwl.c:6-40) and ships no writer
 * and no generator output format.  These keep ensembles made here (the
 * device generator, wl_ensemble_generate) on disk.
 */
#ifndef WL_HOST_H
#define WL_HOST_H

/* Legacy sources include intT.h first, whose profile names and constants
 * (step, smooth, ..., profile, tubedist, lmin, q1, q2, ...) are object-like
 * macros; they are set aside while this header is read and restored after. */
#pragma push_macro("step")
#undef step
#pragma push_macro("smooth")
#undef smooth
#pragma push_macro("quadratic")
#undef quadratic
#pragma push_macro("gaussian")
#undef gaussian
#pragma push_macro("periodic")
#undef periodic
#pragma push_macro("spline")
#undef spline
#pragma push_macro("fixflux")
#undef fixflux
#pragma push_macro("profile")
#undef profile
#pragma push_macro("pi")
#undef pi
#pragma push_macro("tubedist")
#undef tubedist
#pragma push_macro("lmin")
#undef lmin
#pragma push_macro("q1")
#undef q1
#pragma push_macro("q2")
#undef q2
#pragma push_macro("Nspline")
#undef Nspline
#pragma push_macro("verbosity")
#undef verbosity

#include <stdint.h>
#include <vector_types.h> /* float4 */

#ifdef __cplusplus
extern "C" {
#endif

/* the text format getwl reads: per loop Nppl x values, then y, then z (Dim) */
int wlh_putwl(const float4 *worldlines, const char *filename, int Nl, int Nppl, int Dim);

/* Binary ensemble file: a 32-byte little-endian header (magic "WLENSv1",
 * Nl, ppl, the generator seed or 0, 4 values per point) and Nl * ppl float4
 * points, loop-major.  All return 0, or -1 (cannot open, not an ensemble
 * file, wrong shape, short file). */
int wlh_write_ensemble(const char *path, const float4 *loops, int Nl, int ppl, uint64_t seed);
int wlh_ensemble_file_info(const char *path, int *Nl, int *ppl, uint64_t *seed);
int wlh_read_ensemble(const char *path, float4 *loops, int Nl, int ppl);

#ifdef __cplusplus
}
#endif

#pragma pop_macro("step")
#pragma pop_macro("smooth")
#pragma pop_macro("quadratic")
#pragma pop_macro("gaussian")
#pragma pop_macro("periodic")
#pragma pop_macro("spline")
#pragma pop_macro("fixflux")
#pragma pop_macro("profile")
#pragma pop_macro("pi")
#pragma pop_macro("tubedist")
#pragma pop_macro("lmin")
#pragma pop_macro("q1")
#pragma pop_macro("q2")
#pragma pop_macro("Nspline")
#pragma pop_macro("verbosity")

#endif
