// IMesh: the mesh/time-loop driver interface. Same interface as the
// reference's api/fastmesh.h:43-64 (namespace fastmesh), implemented here by
// fastmesh::GpuMesh (gpuMesh.h) on the device path.
#ifndef LFM_FASTMESH_H
#define LFM_FASTMESH_H

#include "inputReader.h"
#include "runTimeManager.h"

namespace fastmesh {

typedef enum fastmesh_solvers { SOLVER_CAAFOAM = 0, SOLVER_M2 = 1, SOLVER_M2PDISS = 2, SOLVER_COUNT } fastmesh_solver_t;

class IMesh {
public:
    virtual ~IMesh() {}
    virtual void initialize() = 0;
    virtual int initializeSolver() = 0;   // 0 on success
    virtual void solve() = 0;
    virtual void finalize() = 0;
    virtual void setInputReader(CInputReader* pInputReader) = 0;
    virtual void setRunTimeManager(IRunTimeManager* pRunTimeManager) = 0;
};

}  // namespace fastmesh

#endif
