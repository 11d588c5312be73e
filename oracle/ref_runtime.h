/* ref_runtime.h -- runtime of the C translation of the reference's hot-path modules.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/f90c.py).  One MPI rank: MPI_SENDRECV to and from the
 * rank itself and MPI_ALLREDUCE are copies; the datatype handles the glue passes are element
 * sizes in bytes.  Fortran `stop` returns control to the glue through longjmp. */
#ifndef WM_REF_RUNTIME_H
#define WM_REF_RUNTIME_H
#include <setjmp.h>
#include <string.h>

extern jmp_buf f90_stop_env;
extern int f90_stopped;

static inline void f90_stop(void)
{
    f90_stopped = 1;
    longjmp(f90_stop_env, 1);
}

static inline void f90_mpi_sendrecv(void *sb, int *scount, int *stype, int *dest, int *stag, void *rb, int *rcount, int *rtype,
                                    int *src, int *rtag, int *comm, int *status, int *err)
{
    (void)dest; (void)stag; (void)rcount; (void)rtype; (void)src; (void)rtag; (void)comm; (void)status;
    memmove(rb, sb, (size_t)(*scount) * (size_t)(*stype));
    *err = 0;
}

static inline void f90_mpi_allreduce(void *s, void *r, int *count, int *type, int *op, int *comm, int *err)
{
    (void)op; (void)comm;
    memmove(r, s, (size_t)(*count) * (size_t)(*type));
    *err = 0;
}
#endif
