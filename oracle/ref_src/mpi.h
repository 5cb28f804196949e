/* Empty stand-in for <mpi.h>: the DG evaluator headers include it
 * (evaluation_dg_laplacian.h:14, evaluation_dg_advect.h:14) but call no MPI
 * function in the code paths used for golden vectors. */
