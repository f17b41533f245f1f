/* Stand-in for the two netCDF calls the per-q stage makes
 * (src/elph/compute_elph_matq.c:149,172,179,212): slices are written to and
 * read from in-memory arrays owned by the oracle harness.  Oracle build only. */
#pragma once
#include <stddef.h>

#define NC_NOERR 0
int nc_put_vara(int ncid, int varid, const size_t* startp, const size_t* countp, const void* op);
int nc_get_vara(int ncid, int varid, const size_t* startp, const size_t* countp, void* ip);
const char* nc_strerror(int ncerr);
