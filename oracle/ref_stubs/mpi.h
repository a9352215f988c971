/* Stand-in MPI type names for compiling the reference's hot-path sources in
 * the oracle harness. No MPI call is made by the code the harness builds; the reference's
 * programs are compiled against them (not linked) to list their symbols. */
#ifndef VGB_STUB_MPI_H
#define VGB_STUB_MPI_H
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Comm;
#define MPI_COMM_WORLD ((MPI_Comm)0)
#endif
