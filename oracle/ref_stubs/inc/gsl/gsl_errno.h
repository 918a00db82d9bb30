/* Stand-in for GSL's error header: the reference's ODE right-hand sides only
 * need the success code. */
#ifndef ORACLE_STUB_GSL_ERRNO_H
#define ORACLE_STUB_GSL_ERRNO_H
#define GSL_SUCCESS 0
#endif
