/* Aborting stand-ins for the LAPACK routines that only non-hot helpers of
 * src/common/blas_lapack.c reference (diagonalize_hermitian,
 * orthogonal_projection).  The per-q stage never calls them.  Oracle build only. */
#include <stdio.h>
#include <stdlib.h>

static void lapack_absent(const char* name)
{
    fprintf(stderr, "LAPACK routine %s is not available in the oracle build\n", name);
    abort();
}
void zheev_(void) { lapack_absent("zheev"); }
void cheev_(void) { lapack_absent("cheev"); }
void dgeqp3_(void) { lapack_absent("dgeqp3"); }
void sgeqp3_(void) { lapack_absent("sgeqp3"); }
void dormqr_(void) { lapack_absent("dormqr"); }
void sormqr_(void) { lapack_absent("sormqr"); }
