/* Minimal single-rank stand-in for <mpi.h>, used ONLY to compile the
 * reference StePS CPU sources (forces.cc, ewald_space.cc, utils.cc, step.cc,
 * friedmann_solver.cc) into the test oracle under oracle/_ref/.
 * Every collective is a no-op because the oracle runs as one rank
 * (numtasks = 1), exactly the configuration in which StePS's own MPI calls
 * degenerate to no-ops. Test infrastructure, never part of the product. */
#ifndef STEPS_ORACLE_MPI_STUB_H
#define STEPS_ORACLE_MPI_STUB_H
typedef int MPI_Status;
typedef int MPI_Datatype;
typedef int MPI_Comm;
#define MPI_FLOAT 1
#define MPI_DOUBLE 2
#define MPI_INT 3
#define MPI_COMM_WORLD 0
static inline int MPI_Bcast(void *b, int c, MPI_Datatype t, int r, MPI_Comm m)
{ (void)b; (void)c; (void)t; (void)r; (void)m; return 0; }
static inline int MPI_Send(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m)
{ (void)b; (void)c; (void)t; (void)d; (void)g; (void)m; return 0; }
static inline int MPI_Recv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m, MPI_Status *st)
{ (void)b; (void)c; (void)t; (void)s; (void)g; (void)m; (void)st; return 0; }
static inline int MPI_Barrier(MPI_Comm m) { (void)m; return 0; }
#endif
