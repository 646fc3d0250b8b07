// fastmesh::GpuMesh: IMesh on one GB300. Reads the case through
// CPolyMeshReaderOF, builds the solver description (lfm::buildSolverCase) and
// runs the time loop of Mesh::solve (reference src/mesh_solver.cpp:172-1076) on
// the device through the C ABI of lfm_gpu.h. Output follows the reference:
// rho, E, p and U are updated in the reader's fields at write times and
// written by the run-time manager with every other AUTO_WRITE field.
//
// A decomposed case (processor0..N-1, what the reference runs as N MPI ranks)
// runs as one process: setPartitionCount(N) before initialize() gives every
// partition its own run-time manager and reader, all partitions advance
// together on the GPU (lfm_partitioned: processor-face halos filled by
// on-device copies), and each partition writes its own processor directory.
#ifndef LFM_GPU_MESH_H
#define LFM_GPU_MESH_H

#include <vector>

#include "fastmesh.h"
#include "meshReader.h"

struct lfm_solver;
struct lfm_partitioned;

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
    // Decomposed case: run partitions processor0..n-1 together (n >= 1;
    // each gets its own run-time manager, so none need be set).
    void setPartitionCount(int n) { m_nPartitions = n; }

    IMeshReader* m_pMeshReader = nullptr;   // the case, or partition 0
    CInputReader* m_pInput = nullptr;
    IRunTimeManager* m_pRunTime = nullptr;  // the case's, or partition 0's

private:
    struct Part {
        IRunTimeManager* runTime = nullptr;
        IMeshReader* reader = nullptr;
        lfm::SolverCase* sc = nullptr;
        lfm_solver* solver = nullptr;   // owned by the mesh, or by m_pPartitioned
    };
    void updateSolution(Part& part);
    void writeFields(Part& part, int timeStep, int indexStartAverage, bool average);
    // haveForces: wall patches (type "wall", in patch order, as the
    // reference's m_nWallBCList) and the records not yet written
    void recordForces(double time);
    void writeForces(bool header);
    std::vector<Part> m_parts;
    std::vector<IRunTimeManager*> m_ownedRunTimes;
    lfm_partitioned* m_pPartitioned = nullptr;
    int m_nPartitions = 0;   // 0: the single case of m_pRunTime
    std::vector<int> m_wallPatches;
    std::vector<double> m_forceTimes;
    std::vector<std::vector<double>> m_forceRows;   // per record: [patch][Fp D, Fv D]
    int m_nPrecision = 0;
    int m_nDevice = 0;
};

}  // namespace fastmesh

#endif
