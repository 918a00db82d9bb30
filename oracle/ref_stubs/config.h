/* Empty autoconf result used when the reference's sources are compiled as an
 * oracle: with no HAVE_CBLAS_H / HAVE_BLAS_H, the reference's matrix.c uses its
 * built-in dgemv/dgemm loops, so no BLAS library is needed. */
