// fastmesh::GpuMesh: IMesh on one GB300. Reads the case through
// CPolyMeshReaderOF, builds the solver description (lfm::buildSolverCase) and
// runs the time loop of Mesh::solve (reference src/mesh_solver.cpp:172-1076) on
// the device through the C ABI of lfm_gpu.h. Output follows the reference:
// rho, E, p and U are updated in the reader's fields at write times and
// written by the run-time manager with every other AUTO_WRITE field.
#ifndef LFM_GPU_MESH_H
#define LFM_GPU_MESH_H

#include <vector>

#include "fastmesh.h"
#include "meshReader.h"

struct lfm_solver;

namespace lfm {
struct SolverCase;
}

namespace fastmesh {

class GpuMesh : public IMesh {
public:
    GpuMesh();
    virtual ~GpuMesh();

    virtual void initialize();
    virtual int initializeSolver();
    virtual void solve();
    virtual void finalize();
    virtual void setInputReader(CInputReader* pInputReader) { m_pInput = pInputReader; }
    virtual void setRunTimeManager(IRunTimeManager* pRunTimeManager) { m_pRunTime = pRunTimeManager; }

    // Arithmetic of the flux kernels (LFM_FP64 or LFM_FP32_BULK).
    void setPrecision(int precision) { m_nPrecision = precision; }
    void setDevice(int device) { m_nDevice = device; }

    IMeshReader* m_pMeshReader = nullptr;
    CInputReader* m_pInput = nullptr;
    IRunTimeManager* m_pRunTime = nullptr;

private:
    void updateSolution();
    // haveForces: wall patches (type "wall", in patch order, as the
    // reference's m_nWallBCList) and the records not yet written
    void recordForces(double time);
    void writeForces(bool header);
    std::vector<int> m_wallPatches;
    std::vector<double> m_forceTimes;
    std::vector<std::vector<double>> m_forceRows;   // per record: [patch][Fp D, Fv D]
    lfm::SolverCase* m_pCase = nullptr;
    lfm_solver* m_pSolver = nullptr;
    int m_nPrecision = 0;
    int m_nDevice = 0;
};

}  // namespace fastmesh

#endif
