/*
 * mpi.h -- declarations only, for compiling the reference's BrickDecomp layout producer
 * (include/brick-mpi.h) into the test-only checker in oracle/_ref without an MPI library.
 *
 * TEST INFRASTRUCTURE ONLY.  BrickDecomp::initialize (brick-mpi.h:322-464) makes no MPI
 * call; the header still names MPI types and functions in its exchange and statistics
 * members.  Those names are declared here and defined nowhere: nothing that calls them is
 * instantiated by oracle/ref_driver.cpp, so a build that tried to use one would fail to link
 * rather than run.
 */
#ifndef BK_ORACLE_MPI_DECLS_H
#define BK_ORACLE_MPI_DECLS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bk_orc_mpi_comm_s *MPI_Comm;
typedef struct bk_orc_mpi_request_s *MPI_Request;
typedef struct bk_orc_mpi_datatype_s *MPI_Datatype;
typedef struct bk_orc_mpi_op_s *MPI_Op;
typedef struct bk_orc_mpi_win_s *MPI_Win;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

extern MPI_Comm bk_orc_mpi_comm_null;
extern MPI_Datatype bk_orc_mpi_char, bk_orc_mpi_double;
extern MPI_Op bk_orc_mpi_sum, bk_orc_mpi_max, bk_orc_mpi_min;
#define MPI_COMM_NULL bk_orc_mpi_comm_null
#define MPI_CHAR bk_orc_mpi_char
#define MPI_DOUBLE bk_orc_mpi_double
#define MPI_SUM bk_orc_mpi_sum
#define MPI_MAX bk_orc_mpi_max
#define MPI_MIN bk_orc_mpi_min

int MPI_Barrier(MPI_Comm comm);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *stats);
int MPI_Win_fence(int assert_, MPI_Win win);
int MPI_Get(void *origin, int ocount, MPI_Datatype otype, int target, long tdisp, int tcount, MPI_Datatype ttype,
            MPI_Win win);
int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);

#ifdef __cplusplus
}
#endif

#endif
