/* Minimal stand-in for <mpi.h> used only to compile the reference solver as
 * the test oracle.  The reference includes mpi.h unconditionally (utils.h:12)
 * but, without -DuseMPI, only names MPI_COMM_WORLD and MPI_Abort in a macro
 * (utils.h:74).  It also relies on <cstring> arriving transitively for
 * strcmp (march.cpp:342). */
#ifndef HAMSTR_ORACLE_MPI_STUB_H
#define HAMSTR_ORACLE_MPI_STUB_H
#include <cstring>
#define MPI_COMM_WORLD 0
static inline int MPI_Abort(int, int) { return 0; }
#endif
