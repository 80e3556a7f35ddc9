/* wl_host.h -- ensemble files of the C host layer (libwlhost.so).
 *
 * No counterpart in the reference, which reads loops only from its text
 * format (getwl, declared in wl_legacy.h, getwl.c:6-40) and ships no writer
 * and no generator output format.  These keep ensembles made here (the
 * device generator, wl_ensemble_generate) on disk.
 */
#ifndef WL_HOST_H
#define WL_HOST_H

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

#endif
