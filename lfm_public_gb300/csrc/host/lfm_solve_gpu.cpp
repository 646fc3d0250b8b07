// lfm_solve_gpu: the reference's lfm_solve (info/lfm_solve.cpp:17-143) on one
// GB300. Run in an OpenFOAM case directory. Same input validation and flags
// (-h, -p/--parallel, -c/--comm_type); invalid input prints a message and
// returns 0, as the reference does. controlDict lfm/doublePrecision false
// selects the FP32-bulk form (FP32 flux, FP64 RK registers) instead of the
// reference's single-precision build. With -p every partition processor0..N-1
// runs in this process on one GPU (LFM_RANK=<r>: partition r alone).
#include <sys/stat.h>

#include <cstdlib>
#include <exception>
#include <iostream>
#include <memory>
#include <string>

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
    // -p: the decomposed case. The reference runs it as one MPI rank per
    // partition (mpirun -np N lfm_solve -p); here one process runs every
    // partition processor0..N-1 on the GPU, or, with LFM_RANK set, that
    // partition alone (which must then have no processor patches).
    int rank = -1, partitions = 0;
    if (input.m_bParallel) {
        const char* r = std::getenv("LFM_RANK");
        if (r) {
            rank = std::atoi(r);
        } else {
            struct stat st;
            while (stat(("processor" + std::to_string(partitions)).c_str(), &st) == 0) ++partitions;
            if (partitions == 0) {
                std::cerr << "-p: no processor0 directory in the case" << std::endl;
                return 1;
            }
        }
    }
    try {
        std::unique_ptr<CRunTimeManagerOF> runTime;
        fastmesh::GpuMesh mesh;
        if (partitions > 0) {
            mesh.setPartitionCount(partitions);
        } else {
            runTime.reset(new CRunTimeManagerOF(rank));
            mesh.setRunTimeManager(runTime.get());
        }
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
