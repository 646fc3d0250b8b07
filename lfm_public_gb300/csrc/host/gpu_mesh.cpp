// fastmesh::GpuMesh: IMesh on the device path (see include/lfm/gpuMesh.h).
//
// The loop follows Mesh::solve (reference src/mesh_solver.cpp:172-1076): while
// the run-time manager runs, one time step (rkOrder stages) is advanced at the
// current deltaT; with adjustTimeStep the next deltaT is compute_dt's minimum,
// otherwise the CFL is reported; time advances; every printInfoFreq steps the
// step, time, CFL / dt (and residuals) are printed; at write times rho, E, p, U
// are stored into the reader's fields (updateSolutionPrimitives,
// src/cfd_v0.cpp:2999-3033) and all AUTO_WRITE fields are written. T and alpha
// are written as read, as the reference does. Post-processing runs on the
// device: haveAverage accumulates pAvg / pRMS after every step from
// tStartAverage on and writes them as fields; haveForces records the wall
// forces at the start and every saveForcesStep steps and appends them to
// ./output/postProcess_Forces_<k> at write times (src/mesh_solver.cpp:253-360,
// 740-756, 828-838, 1081-1123).
#include "gpuMesh.h"

#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
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

void GpuMesh::recordForces(double time) {
    const int D = m_pCase->dim;
    const size_t nw = m_wallPatches.size();
    std::vector<double> fp(nw * (size_t)D), fv(nw * (size_t)D);
    if (lfm_solver_forces(m_pSolver, (int)nw, m_wallPatches.data(), fp.data(), fv.data()) != LFM_OK)
        throw std::runtime_error(std::string("forces: ") + lfm_last_error());
    std::vector<double> row;
    for (size_t i = 0; i < nw; ++i) {
        for (int k = 0; k < D; ++k) row.push_back(fp[i * (size_t)D + (size_t)k]);
        for (int k = 0; k < D; ++k) row.push_back(fv[i * (size_t)D + (size_t)k]);
    }
    m_forceTimes.push_back(time);
    m_forceRows.push_back(row);
}

// output_Forces / postProcForcesOutput (src/mesh_solver.cpp:1081-1123,
// src/cfd_v0.cpp:3254-3275): one file per wall patch.
void GpuMesh::writeForces(bool header) {
    const int D = m_pCase->dim;
    static const char xyz[3] = {'x', 'y', 'z'};
    for (size_t i = 0; i < m_wallPatches.size(); ++i) {
        std::ostringstream name;
        name << "./output/postProcess_Forces_" << i + 1;
        std::ofstream f(name.str(), header ? std::ios::out : std::ios::app);
        if (header) {
            f << std::setw(25) << "time";
            for (int k = 0; k < D; ++k) f << std::setw(25) << "Fp," << xyz[k];
            for (int k = 0; k < D; ++k) f << std::setw(25) << "Fv," << xyz[k];
            for (int k = 0; k < D; ++k) f << std::setw(25) << "Fp," << xyz[k] << " + Fv," << xyz[k];
            f << std::endl;
            continue;
        }
        for (size_t r = 0; r < m_forceTimes.size(); ++r) {
            const double* v = m_forceRows[r].data() + i * 2 * (size_t)D;
            f << std::scientific << std::setprecision(16);
            f << std::setw(25) << m_forceTimes[r];
            for (int k = 0; k < D; ++k) f << std::setw(25) << v[k];
            for (int k = 0; k < D; ++k) f << std::setw(25) << v[D + k];
            for (int k = 0; k < D; ++k) f << std::setw(25) << v[k] + v[D + k];
            f << std::endl;
        }
    }
    if (!header) {
        m_forceTimes.clear();
        m_forceRows.clear();
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
    // pressure statistics from tStartAverage on (src/mesh_solver.cpp:253-270)
    const bool average = m_pInput->m_bHaveAverage;
    const int indexStartAverage = (int)((m_pInput->m_tStartAverage - time) / dt);
    if (average) {
        std::cout << "Statistics will start being computed at t = " << m_pInput->m_tStartAverage
                  << ", at iteration " << indexStartAverage << std::endl;
        m_pMeshReader->createScalarField("pAvg");
        m_pMeshReader->createScalarField("pRMS");
        if (lfm_solver_stats_reset(m_pSolver) != LFM_OK) throw std::runtime_error(lfm_last_error());
    }
    // wall forces: header if the first file is new, then the start record
    // (src/mesh_solver.cpp:341-358, 428)
    const bool forces = m_pInput->m_bHaveForces;
    if (forces) {
        m_wallPatches.clear();
        for (int b = 0; b < m_pMeshReader->getBoundaryCount(); ++b)
            if (m_pMeshReader->getBoundaryType(b) == "wall") m_wallPatches.push_back(b);
        struct stat st;
        if (stat("./output/postProcess_Forces_1", &st) != 0) writeForces(true);
        recordForces(m_pRunTime->getCurrentTime());
    }
    const int saveForces = std::max(1, m_pInput->m_nSaveForcesSteps);
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
        if (average && lfm_solver_stats_accumulate(m_pSolver, timeStep - indexStartAverage) != LFM_OK)
            throw std::runtime_error(lfm_last_error());
        if (forces && timeStep % saveForces == 0) recordForces(time);
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
            const int nAvg = timeStep - indexStartAverage;
            if (average && nAvg >= 1) {   // updateAverages (src/cfd_v0.cpp:2966-2970)
                const size_t nc = (size_t)c.nCells;
                std::vector<double> pa(nc), pr(nc);
                if (lfm_solver_stats_get(m_pSolver, nAvg, pa.data(), pr.data()) != LFM_OK)
                    throw std::runtime_error(lfm_last_error());
                const int iA = m_pMeshReader->getScalarFieldIndex("pAvg");
                const int iR = m_pMeshReader->getScalarFieldIndex("pRMS");
                for (size_t i = 0; i < nc; ++i) {
                    m_pMeshReader->updateScalarField(iA, pa[i], (int)c.cellId[i]);
                    m_pMeshReader->updateScalarField(iR, pr[i], (int)c.cellId[i]);
                }
            }
            if (forces) writeForces(false);
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
