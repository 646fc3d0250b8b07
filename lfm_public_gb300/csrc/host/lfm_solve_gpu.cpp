// lfm_solve_gpu: the reference's lfm_solve (info/lfm_solve.cpp:17-143) on one
// GB300. Run in an OpenFOAM case directory. Same input validation and flags
// (-h, -p/--parallel, -c/--comm_type); invalid input prints a message and
// returns 0, as the reference does. controlDict lfm/doublePrecision false
// selects the FP32-bulk form (FP32 flux, FP64 RK registers) instead of the
// reference's single-precision build. With -p the case is processor<LFM_RANK>.
#include <cstdlib>
#include <exception>
#include <iostream>

#include "gpuMesh.h"
#include "inputReader.h"
#include "lfm_gpu.h"
#include "runTimeManagerOF.h"

int main(int argc, char* argv[]) {
    CInputReader input;
    try {
        if (!input.initialize(argc, argv)) return 0;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 1;
    }
    if (input.m_nSolver < 0 || input.m_nSolver >= fastmesh::SOLVER_COUNT) {
        std::cerr << "unknown solver type: " << input.m_nSolver << std::endl;
        return 0;
    }
    if (input.m_nDimension != 2 && input.m_nDimension != 3) {
        std::cerr << "invalid dimension: " << input.m_nDimension << std::endl;
        return 0;
    }
    if (input.m_nCommType < 0 || input.m_nCommType >= 3) {
        std::cerr << "invalid communication type: " << input.m_nCommType << std::endl;
        return 0;
    }
    if (input.m_nHaloCommType < 0 || input.m_nHaloCommType >= 10) {
        std::cerr << "invalid halo communication type: " << input.m_nHaloCommType << std::endl;
        return 0;
    }
    int rank = -1;
    if (input.m_bParallel) {
        const char* r = std::getenv("LFM_RANK");
        rank = r ? std::atoi(r) : 0;
    }
    try {
        CRunTimeManagerOF runTime(rank);
        fastmesh::GpuMesh mesh;
        mesh.setRunTimeManager(&runTime);
        mesh.setInputReader(&input);
        mesh.setPrecision(input.m_bIsDoublePrecision ? LFM_FP64 : LFM_FP32_BULK);
        const char* dev = std::getenv("LFM_DEVICE");
        mesh.setDevice(dev ? std::atoi(dev) : 0);
        mesh.initialize();
        if (mesh.initializeSolver() != 0) return 0;
        mesh.solve();
        mesh.finalize();
    } catch (const std::exception& e) {
        std::cerr << "lfm_solve_gpu: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
