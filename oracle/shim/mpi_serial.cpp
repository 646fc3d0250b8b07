// Single-rank implementation of the MPI subset in mpi.h (oracle test
// infrastructure; see the header).
#include "mpi.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static size_t typeSize(MPI_Datatype t) {
    switch (t) {
        case MPI_CHAR: return 1;
        case MPI_UNSIGNED_SHORT: return 2;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: case MPI_LOGICAL: return 4;
        case MPI_DOUBLE: case MPI_LONG: return 8;
        default:
            std::fprintf(stderr, "serial MPI: unsupported datatype %d in a collective\n", t);
            std::abort();
    }
}

[[noreturn]] static void unreachable(const char* what) {
    std::fprintf(stderr, "serial MPI: %s is not available on one rank\n", what);
    std::abort();
}

static int g_initialized = 0;

extern "C" {
int MPI_Init(int*, char***) { g_initialized = 1; return 0; }
int MPI_Initialized(int* flag) { *flag = g_initialized; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm, int code) { std::fprintf(stderr, "MPI_Abort(%d)\n", code); std::exit(code); }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return 0; }
int MPI_Comm_split(MPI_Comm comm, int, int, MPI_Comm* out) { *out = comm; return 0; }
int MPI_Comm_group(MPI_Comm, MPI_Group* g) { *g = 1; return 0; }
int MPI_Group_incl(MPI_Group g, int, const int[], MPI_Group* out) { *out = g; return 0; }
int MPI_Group_free(MPI_Group* g) { *g = 0; return 0; }
int MPI_Get_processor_name(char* name, int* len) { std::strcpy(name, "serial"); *len = 6; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Pcontrol(const int, ...) { return 0; }
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) std::memmove(r, s, (size_t)n * typeSize(t));
    return 0;
}
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != r) std::memmove(r, s, (size_t)n * typeSize(t));
    return 0;
}
int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
    if (s != r) std::memmove(r, s, (size_t)n * typeSize(t));
    return 0;
}
int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
    if (s != r) std::memmove(r, s, (size_t)n * typeSize(t));
    return 0;
}
int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { unreachable("MPI_Isend"); }
int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { unreachable("MPI_Irecv"); }
int MPI_Send_init(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { unreachable("MPI_Send_init"); }
int MPI_Recv_init(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { unreachable("MPI_Recv_init"); }
int MPI_Start(MPI_Request*) { unreachable("MPI_Start"); }
int MPI_Startall(int n, MPI_Request[]) { if (n) unreachable("MPI_Startall"); return 0; }
int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
int MPI_Waitall(int, MPI_Request[], MPI_Status*) { return 0; }
int MPI_Testall(int, MPI_Request[], int* flag, MPI_Status*) { *flag = 1; return 0; }
int MPI_Type_create_struct(int, const int[], const MPI_Aint[], const MPI_Datatype[], MPI_Datatype* out) {
    *out = 100; return 0;
}
int MPI_Type_create_resized(MPI_Datatype in, MPI_Aint, MPI_Aint, MPI_Datatype* out) { *out = in; return 0; }
int MPI_Type_commit(MPI_Datatype*) { return 0; }
int MPI_Win_create(void*, MPI_Aint, int, MPI_Info, MPI_Comm, MPI_Win* w) { *w = 1; return 0; }
int MPI_Win_free(MPI_Win* w) { *w = 0; return 0; }
int MPI_Win_post(MPI_Group, int, MPI_Win) { return 0; }
int MPI_Win_start(MPI_Group, int, MPI_Win) { return 0; }
int MPI_Win_complete(MPI_Win) { return 0; }
int MPI_Win_wait(MPI_Win) { return 0; }
int MPI_Win_lock(int, int, int, MPI_Win) { return 0; }
int MPI_Win_lock_all(int, MPI_Win) { return 0; }
int MPI_Get(void*, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win) { unreachable("MPI_Get"); }
int MPI_Rget(void*, int, MPI_Datatype, int, MPI_Aint, int, MPI_Datatype, MPI_Win, MPI_Request*) {
    unreachable("MPI_Rget");
}
int MPI_Dist_graph_create_adjacent(MPI_Comm comm, int, const int[], const int[], int, const int[], const int[],
                                   MPI_Info, int, MPI_Comm* out) { *out = comm; return 0; }
int MPI_Dist_graph_neighbors(MPI_Comm, int, int[], int[], int, int[], int[]) { return 0; }
}
