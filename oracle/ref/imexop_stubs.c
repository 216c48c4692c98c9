/*
 * Oracle test infrastructure: stand-ins for the symbols that
 * suzerain/blas_et_al/blasext.c references but that the rholut_imexop path of
 * the oracle's reference build never calls (single-precision and real BLAS
 * wrappers, and the fixed-bandwidth kernels the reference generates with
 * Boost.Preprocessor).  Each reports the call and aborts.  This file includes
 * no reference header, so the stand-ins need no signatures.
 */
#include <stdio.h>
#include <stdlib.h>

static void oracle_ref_unreachable(const char *name)
{
    fprintf(stderr, "oracle reference build: %s is not part of this build\n", name);
    abort();
}

#define ORACLE_STUB(name) void name(void); void name(void) { oracle_ref_unreachable(#name); }
ORACLE_STUB(suzerain_blas_caxpby)
ORACLE_STUB(suzerain_blas_caxpy)
ORACLE_STUB(suzerain_blas_cgbmv_s_c_external)
ORACLE_STUB(suzerain_blas_csbmv_s_c_external)
ORACLE_STUB(suzerain_blas_daxpby)
ORACLE_STUB(suzerain_blas_dgbmv_external)
ORACLE_STUB(suzerain_blas_dsbmv_external)
ORACLE_STUB(suzerain_blas_saxpby)
ORACLE_STUB(suzerain_blas_saxpy)
ORACLE_STUB(suzerain_blas_sgbmv_external)
ORACLE_STUB(suzerain_blas_ssbmv_external)
ORACLE_STUB(suzerain_blas_zgbmv_d_z_external)
ORACLE_STUB(suzerain_blas_zsbmv_d_z_external)
ORACLE_STUB(suzerain_gbdddddmv_d)
ORACLE_STUB(suzerain_gbdddddmv_ddz)
ORACLE_STUB(suzerain_gbdddddmv_s)
ORACLE_STUB(suzerain_gbdddddmv_scc)
ORACLE_STUB(suzerain_gbdddddmv_ssc)
ORACLE_STUB(suzerain_gbddddmv_d)
ORACLE_STUB(suzerain_gbddddmv_ddz)
ORACLE_STUB(suzerain_gbddddmv_s)
ORACLE_STUB(suzerain_gbddddmv_scc)
ORACLE_STUB(suzerain_gbddddmv_ssc)
ORACLE_STUB(suzerain_gbdddmv_d)
ORACLE_STUB(suzerain_gbdddmv_ddz)
ORACLE_STUB(suzerain_gbdddmv_s)
ORACLE_STUB(suzerain_gbdddmv_scc)
ORACLE_STUB(suzerain_gbdddmv_ssc)
ORACLE_STUB(suzerain_gbddmv_d)
ORACLE_STUB(suzerain_gbddmv_ddz)
ORACLE_STUB(suzerain_gbddmv_s)
ORACLE_STUB(suzerain_gbddmv_scc)
ORACLE_STUB(suzerain_gbddmv_ssc)
ORACLE_STUB(suzerain_gbdmv_d)
ORACLE_STUB(suzerain_gbdmv_ddz)
ORACLE_STUB(suzerain_gbdmv_s)
ORACLE_STUB(suzerain_gbdmv_scc)
ORACLE_STUB(suzerain_gbdmv_ssc)
ORACLE_STUB(suzerain_lapack_clangb)
ORACLE_STUB(suzerain_lapack_slangb)
