// fastmesh::GpuMesh: IMesh on the device path (see include/lfm/gpuMesh.h).
//
// The loop follows Mesh::solve (reference src/mesh_solver.cpp:172-1076): while
// the run-time manager runs, one time step (rkOrder stages) is advanced at the
// current deltaT; with adjustTimeStep the next deltaT is compute_dt's minimum,
// otherwise the CFL is reported; time advances; every printInfoFreq steps the
// step, time, CFL / dt (and residuals) are printed; at write times rho, E, p, U
// are stored into the reader's fields (updateSolutionPrimitives,
// src/cfd_v0.cpp:2999-3033) and all AUTO_WRITE fields are written. T and alpha
// are written as read, as the reference does.
#include "gpuMesh.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "case_setup.h"
#include "lfm_gpu.h"
#include "polyMeshReaderOF.h"

namespace fastmesh {

GpuMesh::GpuMesh() {}

GpuMesh::~GpuMesh() {
    finalize();
    delete m_pMeshReader;
    m_pMeshReader = nullptr;
}

void GpuMesh::initialize() {
    if (!m_pRunTime) throw std::runtime_error("GpuMesh: no run-time manager");
    std::cout << "read mesh files..." << std::endl;
    m_pMeshReader = new CPolyMeshReaderOF(m_pRunTime->getRunPointer());
}

int GpuMesh::initializeSolver() {
    if (!m_pMeshReader || !m_pInput) return 1;
    lfm::CaseParams p;
    p.solver = m_pInput->m_nSolver;
    p.dimension = m_pInput->m_nDimension;
    p.rkOrder = m_pInput->m_nRkStepCount;
    p.minmod = m_pInput->m_bMinmodInterpolation;
    p.laminar = m_pInput->m_bisLaminar;
    p.residuals = m_pInput->m_bHaveResidual;
    p.pInf = m_pInput->m_dPInf;
    p.TInf = m_pInput->m_dTInf;
    for (int k = 0; k < 3; ++k) p.UInf[k] = m_pInput->m_dUInf[k];
    p.Ls = m_pInput->m_dLs;
    p.mach = m_pInput->m_dMach;
    p.kSponge = m_pInput->m_dK;
    p.Cp = m_pInput->m_dCp;
    p.molWeight = m_pInput->m_dMolWeight;
    p.mu = m_pInput->m_dMu0;
    p.Pr = m_pInput->m_dPrandtl;
    if (!p.laminar) {
        std::cerr << "Only laminar simulations run on the device path" << std::endl;
        return 2;
    }
    try {
        m_pCase = new lfm::SolverCase(lfm::buildSolverCase(*m_pMeshReader, p));
    } catch (const std::exception& e) {
        std::cerr << "solver setup failed: " << e.what() << std::endl;
        return 3;
    }
    lfm_solver_desc desc;
    lfm::describeSolverCase(*m_pCase, &desc);
    lfm_solver_opts opts{m_nPrecision, m_nDevice, 0};
    if (lfm_solver_create(&desc, &opts, &m_pSolver) != LFM_OK) {
        std::cerr << "device solver: " << lfm_last_error() << std::endl;
        return 4;
    }
    return 0;
}

void GpuMesh::updateSolution() {
    const lfm::SolverCase& c = *m_pCase;
    const int D = c.dim;
    const size_t nc = (size_t)c.nCells;
    std::vector<double> q((size_t)c.nq * nc);
    if (lfm_solver_get_state(m_pSolver, q.data()) != LFM_OK)
        throw std::runtime_error(std::string("device state: ") + lfm_last_error());
    const int iRho = m_pMeshReader->getScalarFieldIndex("rho");
    const int iE = m_pMeshReader->getScalarFieldIndex("E");
    const int iP = m_pMeshReader->getScalarFieldIndex("p");
    const int iU = m_pMeshReader->getVectorFieldIndex("U");
    const double gm1 = c.gamma - 1.0;
    double uvw[3] = {0, 0, 0};
    for (size_t i = 0; i < nc; ++i) {
        const int cell = (int)c.cellId[i];
        const double r = q[i];
        double um2 = 0;
        for (int d = 0; d < D; ++d) {
            uvw[d] = q[(size_t)(d + 1) * nc + i] / r;
            um2 += uvw[d] * uvw[d];
        }
        const double E = q[(size_t)(D + 1) * nc + i] / r;
        const double pr = r * gm1 * (E - 0.5 * um2);
        m_pMeshReader->updateScalarField(iRho, r, cell);
        m_pMeshReader->updateScalarField(iE, E, cell);
        m_pMeshReader->updateScalarField(iP, pr, cell);
        m_pMeshReader->updateVectorField(iU, uvw, cell);
    }
}

void GpuMesh::solve() {
    if (!m_pSolver) throw std::runtime_error("GpuMesh::solve before initializeSolver");
    const lfm::SolverCase& c = *m_pCase;
    std::cout << "\n~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\n"
              << "CFD solver: caafoam on " << (m_nPrecision == LFM_FP32_BULK ? "GB300 (FP32 flux, FP64 RK)"
                                                                            : "GB300 (FP64)")
              << "\n    - cells        : " << c.nCells << "\n    - flux faces   : " << c.nFaces
              << "\n~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\n";
    static const char* schemes[] = {"M1", "M2", "M2 AUSM"};
    std::cout << "Running with " << schemes[c.solver] << " discretization\nLaminar simulation\n" << std::endl;

    m_pMeshReader->createScalarField("rho");
    m_pMeshReader->createScalarField("E");
    m_pMeshReader->createScalarField("p");
    static const char* resNames[] = {"uRES", "vRES", "wRES"};
    const bool saveRes = m_pInput->m_bHaveResidual && m_pInput->m_bSaveResiduals;
    if (saveRes) {
        m_pMeshReader->createScalarField("rhoRES");
        m_pMeshReader->createScalarField("eRES");
        for (int d = 0; d < c.dim; ++d) m_pMeshReader->createScalarField(resNames[d]);
    }
    if (m_pInput->m_bSaveBlendFactor) {
        const int idx = m_pMeshReader->createScalarField("sigma0");
        for (size_t i = 0; i < c.cellId.size(); ++i)
            m_pMeshReader->updateScalarField(idx, c.sponge[i], (int)c.cellId[i]);
    }
    if (m_pInput->m_bSaveRank) {
        const int idx = m_pMeshReader->createScalarField("rank");
        for (int i = m_pMeshReader->getCellCount() - 1; i >= 0; --i) m_pMeshReader->updateScalarField(idx, 0.0, i);
    }
    if (m_pInput->m_bSaveCellOrder) {
        const int idx = m_pMeshReader->createScalarField("cellOrder");
        for (int i = m_pMeshReader->getCellCount() - 1; i >= 0; --i)
            m_pMeshReader->updateScalarField(idx, (double)i, i);
    }

    double dt = m_pRunTime->getDeltaTime();
    double time = m_pRunTime->getCurrentTime();
    const double tEnd = m_pRunTime->getEndTime();
    double cflMax = m_pInput->m_dCFLMax;
    int timeStep = 0;
    double rkLoop = 0.0, outputTime = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<double> res((size_t)c.nq, 0.0);
    while (m_pRunTime->isRunning()) {
        dt = m_pRunTime->getDeltaTime();
        const auto a = std::chrono::steady_clock::now();
        if (lfm_solver_step(m_pSolver, 1, dt) != LFM_OK || lfm_solver_sync(m_pSolver) != LFM_OK)
            throw std::runtime_error(std::string("time step failed: ") + lfm_last_error());
        rkLoop += std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        const bool print = ((timeStep + 1) % std::max(1, m_pInput->m_nPrintInfoFrequency) == 0) ||
                           (time + dt >= tEnd);
        if (m_pRunTime->isAdjustDeltaTime()) {
            double ndt = dt;
            if (lfm_solver_min_dt(m_pSolver, cflMax, &ndt) != LFM_OK)
                throw std::runtime_error(lfm_last_error());
            m_pRunTime->setDeltaTime(ndt);
        } else if (print) {
            if (lfm_solver_cfl(m_pSolver, dt, &cflMax) != LFM_OK) throw std::runtime_error(lfm_last_error());
        }
        m_pRunTime->advanceTime();
        time += dt;
        ++timeStep;
        if (print) {
            std::printf("Time step: %d     Time: %.10g", timeStep, time);
            if (m_pRunTime->isAdjustDeltaTime())
                std::printf("       dt: %.10g", m_pRunTime->getDeltaTime());
            else
                std::printf("      CFL: %.10g", cflMax);
            if (m_pInput->m_bHaveResidual && lfm_solver_residual(m_pSolver, res.data()) == LFM_OK) {
                std::printf("     Residuals: ");
                for (double r : res) std::printf("%25.15e", std::sqrt(r));
            }
            std::printf("\n\n");
        }
        if (m_pRunTime->isWriteTime()) {
            const auto b = std::chrono::steady_clock::now();
            if (saveRes) {
                // updateSolutionResidual (src/cfd_v0.cpp:2973-2993)
                const size_t nc = (size_t)c.nCells;
                std::vector<double> cr((size_t)c.nq * nc);
                if (lfm_solver_cell_residual(m_pSolver, cr.data()) != LFM_OK)
                    throw std::runtime_error(lfm_last_error());
                const int iR = m_pMeshReader->getScalarFieldIndex("rhoRES");
                const int iE = m_pMeshReader->getScalarFieldIndex("eRES");
                for (size_t i = 0; i < nc; ++i) {
                    const int cell = (int)c.cellId[i];
                    m_pMeshReader->updateScalarField(iR, cr[i], cell);
                    for (int d = 0; d < c.dim; ++d)
                        m_pMeshReader->updateScalarField(m_pMeshReader->getScalarFieldIndex(resNames[d]),
                                                         cr[(size_t)(d + 1) * nc + i], cell);
                    m_pMeshReader->updateScalarField(iE, cr[(size_t)(c.dim + 1) * nc + i], cell);
                }
            }
            updateSolution();
            m_pRunTime->writeResults();
            outputTime += std::chrono::duration<double>(std::chrono::steady_clock::now() - b).count();
        }
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\nTotal Time [1 GPU]\n");
    std::printf("[    ][%.5lf]: Complete Simulation\n", total);
    std::printf("\t[%.2lf %%] / [%.5lf]: Rk Loop\n", total > 0 ? 100 * rkLoop / total : 0.0, rkLoop);
    std::printf("\t[%.2lf %%] / [%.5lf]: Output Time\n", total > 0 ? 100 * outputTime / total : 0.0, outputTime);
    if (rkLoop > 0)
        std::printf("Cell-RK-stage updates/s: %.6e\n", (double)c.nCells * c.rkOrder * timeStep / rkLoop);
    std::printf("\nSimulation finished successfully.\n\n");
}

void GpuMesh::finalize() {
    if (m_pSolver) {
        lfm_solver_destroy(m_pSolver);
        m_pSolver = nullptr;
    }
    delete m_pCase;
    m_pCase = nullptr;
}

}  // namespace fastmesh
