/* Minimal stand-in for the GSL status codes periodic.c tests
 * (periodic.c:24, 142-149).  Test infrastructure for oracle/_ref only; GSL is
 * not installed.  The values are GSL's public ones. */
#ifndef WLREF_GSL_ERRNO_H
#define WLREF_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_FAILURE (-1)
#endif
