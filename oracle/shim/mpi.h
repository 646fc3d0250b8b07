/* Single-rank MPI subset for building the reference solver as the oracle.
 *
 * Test infrastructure only: the reference's src/*.cpp include "mpi.h"; this
 * header lets them compile and run as one rank with no MPI library installed.
 * Every collective is the identity on one rank; point-to-point and one-sided
 * calls are never reached on one rank (the reference skips them when it has
 * no MPI neighbours, src/cfd_v0.cpp:437-439) and abort if they are. */
#ifndef LFM_ORACLE_SERIAL_MPI_H
#define LFM_ORACLE_SERIAL_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Win;
typedef int MPI_Group;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_MAJOR_VERSION 3
#define MPI_COMM_WORLD 1
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_MODE_NOCHECK 1024
#define MPI_MODE_NOPUT 4096
#define MPI_LOCK_SHARED 2
#define MPI_UNWEIGHTED ((int*)0)

#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_UNSIGNED 3
#define MPI_UNSIGNED_SHORT 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 6
#define MPI_LOGICAL 7
#define MPI_LONG 8

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

int MPI_Init(int* argc, char*** argv);
int MPI_Initialized(int* flag);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out);
int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* out);
int MPI_Group_free(MPI_Group* group);
int MPI_Get_processor_name(char* name, int* len);
int MPI_Barrier(MPI_Comm comm);
int MPI_Pcontrol(const int level, ...);
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Gather(const void* send, int scount, MPI_Datatype stype, void* recv, int rcount, MPI_Datatype rtype,
               int root, MPI_Comm comm);
int MPI_Allgather(const void* send, int scount, MPI_Datatype stype, void* recv, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Send_init(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
                  MPI_Request* req);
int MPI_Recv_init(void* buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Start(MPI_Request* req);
int MPI_Startall(int n, MPI_Request reqs[]);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int n, MPI_Request reqs[], MPI_Status* statuses);
int MPI_Testall(int n, MPI_Request reqs[], int* flag, MPI_Status* statuses);
int MPI_Type_create_struct(int n, const int lens[], const MPI_Aint disps[], const MPI_Datatype types[],
                           MPI_Datatype* out);
int MPI_Type_create_resized(MPI_Datatype in, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* out);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Win_create(void* base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, MPI_Win* win);
int MPI_Win_free(MPI_Win* win);
int MPI_Win_post(MPI_Group group, int assert_, MPI_Win win);
int MPI_Win_start(MPI_Group group, int assert_, MPI_Win win);
int MPI_Win_complete(MPI_Win win);
int MPI_Win_wait(MPI_Win win);
int MPI_Win_lock(int type, int rank, int assert_, MPI_Win win);
int MPI_Win_lock_all(int assert_, MPI_Win win);
int MPI_Get(void* origin, int ocount, MPI_Datatype otype, int target, MPI_Aint disp, int tcount,
            MPI_Datatype ttype, MPI_Win win);
int MPI_Rget(void* origin, int ocount, MPI_Datatype otype, int target, MPI_Aint disp, int tcount,
             MPI_Datatype ttype, MPI_Win win, MPI_Request* req);
int MPI_Dist_graph_create_adjacent(MPI_Comm comm, int indegree, const int sources[], const int sweights[],
                                   int outdegree, const int dests[], const int dweights[], MPI_Info info,
                                   int reorder, MPI_Comm* out);
int MPI_Dist_graph_neighbors(MPI_Comm comm, int maxin, int sources[], int sweights[], int maxout, int dests[],
                             int dweights[]);

#ifdef __cplusplus
}
#endif
#endif
