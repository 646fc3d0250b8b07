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
// 740-756, 828-838, 1081-1123). A decomposed case runs all its partitions in
// this process: the reductions the reference does over MPI ranks (CFL and dt
// minimum, residual and force sums) run over the partitions.
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
#include "runTimeManagerOF.h"

namespace fastmesh {

namespace {

void check(int rc, const char* what) {
    if (rc != LFM_OK) throw std::runtime_error(std::string(what) + ": " + lfm_last_error());
}

}  // namespace

GpuMesh::GpuMesh() {}

GpuMesh::~GpuMesh() {
    finalize();
    for (Part& p : m_parts) delete p.reader;
    m_parts.clear();
    m_pMeshReader = nullptr;
    for (IRunTimeManager* rt : m_ownedRunTimes) delete rt;
    m_ownedRunTimes.clear();
}

void GpuMesh::initialize() {
    std::cout << "read mesh files..." << std::endl;
    if (m_nPartitions <= 0) {
        if (!m_pRunTime) throw std::runtime_error("GpuMesh: no run-time manager");
        Part p;
        p.runTime = m_pRunTime;
        p.reader = new CPolyMeshReaderOF(m_pRunTime->getRunPointer());
        m_parts.push_back(p);
    } else {
        for (int r = 0; r < m_nPartitions; ++r) {
            Part p;
            p.runTime = new CRunTimeManagerOF(r);
            m_ownedRunTimes.push_back(p.runTime);
            p.reader = new CPolyMeshReaderOF(p.runTime->getRunPointer());
            m_parts.push_back(p);
        }
        m_pRunTime = m_parts[0].runTime;
    }
    m_pMeshReader = m_parts[0].reader;
}

int GpuMesh::initializeSolver() {
    if (m_parts.empty() || !m_pInput) return 1;
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
    try {
        if (m_nPartitions <= 0) {
            m_parts[0].sc = new lfm::SolverCase(lfm::buildSolverCase(*m_parts[0].reader, p));
        } else {
            std::vector<IMeshReader*> readers;
            for (Part& q : m_parts) readers.push_back(q.reader);
            std::vector<lfm::SolverCase> cases = lfm::buildPartitionCases(readers, p);
            for (size_t k = 0; k < m_parts.size(); ++k) m_parts[k].sc = new lfm::SolverCase(std::move(cases[k]));
        }
    } catch (const std::exception& e) {
        std::cerr << "solver setup failed: " << e.what() << std::endl;
        return 3;
    }
    lfm_solver_opts opts{m_nPrecision, m_nDevice, 0};
    std::vector<lfm_solver_desc> descs(m_parts.size());
    for (size_t k = 0; k < m_parts.size(); ++k) lfm::describeSolverCase(*m_parts[k].sc, &descs[k]);
    if (m_nPartitions <= 0) {
        if (lfm_solver_create(&descs[0], &opts, &m_parts[0].solver) != LFM_OK) {
            std::cerr << "device solver: " << lfm_last_error() << std::endl;
            return 4;
        }
        return 0;
    }
    std::vector<const lfm_solver_desc*> dp;
    for (auto& d : descs) dp.push_back(&d);
    if (lfm_partitioned_create(dp.data(), (int)dp.size(), &opts, &m_pPartitioned) != LFM_OK) {
        std::cerr << "device solver: " << lfm_last_error() << std::endl;
        return 4;
    }
    for (size_t k = 0; k < m_parts.size(); ++k)
        check(lfm_partitioned_solver(m_pPartitioned, (int)k, &m_parts[k].solver), "partition solver");
    return 0;
}

void GpuMesh::updateSolution(Part& part) {
    const lfm::SolverCase& c = *part.sc;
    IMeshReader* rd = part.reader;
    const int D = c.dim;
    const size_t nc = (size_t)c.nCells;
    std::vector<double> q((size_t)c.nq * nc);
    check(lfm_solver_get_state(part.solver, q.data()), "device state");
    const int iRho = rd->getScalarFieldIndex("rho");
    const int iE = rd->getScalarFieldIndex("E");
    const int iP = rd->getScalarFieldIndex("p");
    const int iU = rd->getVectorFieldIndex("U");
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
        rd->updateScalarField(iRho, r, cell);
        rd->updateScalarField(iE, E, cell);
        rd->updateScalarField(iP, pr, cell);
        rd->updateVectorField(iU, uvw, cell);
    }
}

// Fields of one partition at a write time: residuals (updateSolutionResidual,
// src/cfd_v0.cpp:2973-2993), rho, E, p, U, and pAvg / pRMS (updateAverages,
// src/cfd_v0.cpp:2966-2970).
void GpuMesh::writeFields(Part& part, int timeStep, int indexStartAverage, bool average) {
    static const char* resNames[] = {"uRES", "vRES", "wRES"};
    const lfm::SolverCase& c = *part.sc;
    IMeshReader* rd = part.reader;
    const size_t nc = (size_t)c.nCells;
    if (m_pInput->m_bHaveResidual && m_pInput->m_bSaveResiduals) {
        std::vector<double> cr((size_t)c.nq * nc);
        check(lfm_solver_cell_residual(part.solver, cr.data()), "cell residual");
        const int iR = rd->getScalarFieldIndex("rhoRES");
        const int iE = rd->getScalarFieldIndex("eRES");
        for (size_t i = 0; i < nc; ++i) {
            const int cell = (int)c.cellId[i];
            rd->updateScalarField(iR, cr[i], cell);
            for (int d = 0; d < c.dim; ++d)
                rd->updateScalarField(rd->getScalarFieldIndex(resNames[d]), cr[(size_t)(d + 1) * nc + i], cell);
            rd->updateScalarField(iE, cr[(size_t)(c.dim + 1) * nc + i], cell);
        }
    }
    updateSolution(part);
    const int nAvg = timeStep - indexStartAverage;
    if (average && nAvg >= 1) {
        std::vector<double> pa(nc), pr(nc);
        check(lfm_solver_stats_get(part.solver, nAvg, pa.data(), pr.data()), "statistics");
        const int iA = rd->getScalarFieldIndex("pAvg");
        const int iR = rd->getScalarFieldIndex("pRMS");
        for (size_t i = 0; i < nc; ++i) {
            rd->updateScalarField(iA, pa[i], (int)c.cellId[i]);
            rd->updateScalarField(iR, pr[i], (int)c.cellId[i]);
        }
    }
}

// postProcForces over every partition: the sum over the partitions of each
// wall patch's force (the reference's MPI_Allreduce, src/cfd_v0.cpp:3243-3244).
void GpuMesh::recordForces(double time) {
    const int D = m_parts[0].sc->dim;
    const size_t nw = m_wallPatches.size();
    std::vector<double> fp(nw * (size_t)D), fv(nw * (size_t)D), sp(nw * (size_t)D, 0.0), sv(nw * (size_t)D, 0.0);
    for (Part& part : m_parts) {
        check(lfm_solver_forces(part.solver, (int)nw, m_wallPatches.data(), fp.data(), fv.data()), "forces");
        for (size_t k = 0; k < fp.size(); ++k) {
            sp[k] += fp[k];
            sv[k] += fv[k];
        }
    }
    std::vector<double> row;
    for (size_t i = 0; i < nw; ++i) {
        for (int k = 0; k < D; ++k) row.push_back(sp[i * (size_t)D + (size_t)k]);
        for (int k = 0; k < D; ++k) row.push_back(sv[i * (size_t)D + (size_t)k]);
    }
    m_forceTimes.push_back(time);
    m_forceRows.push_back(row);
}

// output_Forces / postProcForcesOutput (src/mesh_solver.cpp:1081-1123,
// src/cfd_v0.cpp:3254-3275): one file per wall patch.
void GpuMesh::writeForces(bool header) {
    const int D = m_parts[0].sc->dim;
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
    if (m_parts.empty() || !m_parts[0].solver) throw std::runtime_error("GpuMesh::solve before initializeSolver");
    const lfm::SolverCase& c0 = *m_parts[0].sc;
    int64_t cells = 0, faces = 0;
    for (Part& p : m_parts) {
        cells += p.sc->nCells;
        faces += p.sc->nFaces;
    }
    std::cout << "\n~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\n"
              << "CFD solver: caafoam on " << (m_nPrecision == LFM_FP32_BULK ? "GB300 (FP32 flux, FP64 RK)"
                                                                            : "GB300 (FP64)")
              << "\n    - partitions   : " << m_parts.size() << "\n    - cells        : " << cells
              << "\n    - flux faces   : " << faces
              << "\n~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\n";
    static const char* schemes[] = {"M1", "M2", "M2 AUSM"};
    std::cout << "Running with " << schemes[c0.solver] << " discretization\n"
              << (c0.smagC.empty() ? "Laminar simulation" : "LES simulation (Smagorinsky)") << "\n" << std::endl;

    static const char* resNames[] = {"uRES", "vRES", "wRES"};
    const bool saveRes = m_pInput->m_bHaveResidual && m_pInput->m_bSaveResiduals;
    const bool average = m_pInput->m_bHaveAverage;
    for (size_t rank = 0; rank < m_parts.size(); ++rank) {
        Part& part = m_parts[rank];
        IMeshReader* rd = part.reader;
        const lfm::SolverCase& c = *part.sc;
        if (average) {
            rd->createScalarField("pAvg");
            rd->createScalarField("pRMS");
            check(lfm_solver_stats_reset(part.solver), "statistics");
        }
        rd->createScalarField("rho");
        rd->createScalarField("E");
        rd->createScalarField("p");
        if (saveRes) {
            rd->createScalarField("rhoRES");
            rd->createScalarField("eRES");
            for (int d = 0; d < c.dim; ++d) rd->createScalarField(resNames[d]);
        }
        if (m_pInput->m_bSaveBlendFactor) {
            const int idx = rd->createScalarField("sigma0");
            for (size_t i = 0; i < c.cellId.size(); ++i) rd->updateScalarField(idx, c.sponge[i], (int)c.cellId[i]);
        }
        if (m_pInput->m_bSaveRank) {   // the partition stands for the reference's MPI rank
            const int idx = rd->createScalarField("rank");
            for (int i = rd->getCellCount() - 1; i >= 0; --i) rd->updateScalarField(idx, (double)rank, i);
        }
        if (m_pInput->m_bSaveCellOrder) {
            const int idx = rd->createScalarField("cellOrder");
            for (int i = rd->getCellCount() - 1; i >= 0; --i) rd->updateScalarField(idx, (double)i, i);
        }
    }

    double dt = m_pRunTime->getDeltaTime();
    double time = m_pRunTime->getCurrentTime();
    const double tEnd = m_pRunTime->getEndTime();
    // pressure statistics from tStartAverage on (src/mesh_solver.cpp:253-270)
    const int indexStartAverage = (int)((m_pInput->m_tStartAverage - time) / dt);
    if (average)
        std::cout << "Statistics will start being computed at t = " << m_pInput->m_tStartAverage
                  << ", at iteration " << indexStartAverage << std::endl;
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
    std::vector<double> res((size_t)c0.nq, 0.0), resPart((size_t)c0.nq, 0.0);
    while (m_pRunTime->isRunning()) {
        dt = m_pRunTime->getDeltaTime();
        const auto a = std::chrono::steady_clock::now();
        if (m_pPartitioned) {
            check(lfm_partitioned_step(m_pPartitioned, 1, dt), "time step");
            check(lfm_partitioned_sync(m_pPartitioned), "time step");
        } else {
            check(lfm_solver_step(m_parts[0].solver, 1, dt), "time step");
            check(lfm_solver_sync(m_parts[0].solver), "time step");
        }
        rkLoop += std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        if (m_pRunTime->isAdjustDeltaTime()) {   // compute_dt + MPI_Allreduce(MIN)
            // the reduction writes the new dt into the variable the step's
            // time is then advanced by (src/mesh_solver.cpp:705-716, 733)
            double ndt = 0.0;
            for (size_t k = 0; k < m_parts.size(); ++k) {
                double d = dt;
                check(lfm_solver_min_dt(m_parts[k].solver, cflMax, &d), "compute_dt");
                ndt = k == 0 ? d : std::min(ndt, d);
            }
            for (Part& p : m_parts) p.runTime->setDeltaTime(ndt);
            dt = ndt;
        }
        const bool print = ((timeStep + 1) % std::max(1, m_pInput->m_nPrintInfoFrequency) == 0) ||
                           (time + dt >= tEnd);
        if (!m_pRunTime->isAdjustDeltaTime() && print) {   // compute_cfl + MPI_Allreduce(MAX)
            for (size_t k = 0; k < m_parts.size(); ++k) {
                double cfl = 0.0;
                check(lfm_solver_cfl(m_parts[k].solver, dt, &cfl), "compute_cfl");
                cflMax = k == 0 ? cfl : std::max(cflMax, cfl);
            }
        }
        for (Part& p : m_parts) p.runTime->advanceTime();
        time += dt;
        ++timeStep;
        if (average)
            for (Part& p : m_parts) check(lfm_solver_stats_accumulate(p.solver, timeStep - indexStartAverage), "statistics");
        if (forces && timeStep % saveForces == 0) recordForces(time);
        if (print) {
            std::printf("Time step: %d     Time: %.10g", timeStep, time);
            if (m_pRunTime->isAdjustDeltaTime())
                std::printf("       dt: %.10g", m_pRunTime->getDeltaTime());
            else
                std::printf("      CFL: %.10g", cflMax);
            if (m_pInput->m_bHaveResidual) {   // residual sums over the partitions (MPI_Reduce SUM)
                std::fill(res.begin(), res.end(), 0.0);
                bool ok = true;
                for (Part& p : m_parts) {
                    ok = ok && lfm_solver_residual(p.solver, resPart.data()) == LFM_OK;
                    for (size_t v = 0; v < res.size(); ++v) res[v] += resPart[v];
                }
                if (ok) {
                    std::printf("     Residuals: ");
                    for (double r : res) std::printf("%25.15e", std::sqrt(r));
                }
            }
            std::printf("\n\n");
        }
        if (m_pRunTime->isWriteTime()) {
            const auto b = std::chrono::steady_clock::now();
            for (Part& p : m_parts) writeFields(p, timeStep, indexStartAverage, average);
            if (forces) writeForces(false);
            for (Part& p : m_parts) p.runTime->writeResults();
            outputTime += std::chrono::duration<double>(std::chrono::steady_clock::now() - b).count();
        }
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~~\nTotal Time [1 GPU]\n");
    std::printf("[    ][%.5lf]: Complete Simulation\n", total);
    std::printf("\t[%.2lf %%] / [%.5lf]: Rk Loop\n", total > 0 ? 100 * rkLoop / total : 0.0, rkLoop);
    std::printf("\t[%.2lf %%] / [%.5lf]: Output Time\n", total > 0 ? 100 * outputTime / total : 0.0, outputTime);
    if (rkLoop > 0)
        std::printf("Cell-RK-stage updates/s: %.6e\n", (double)cells * c0.rkOrder * timeStep / rkLoop);
    std::printf("\nSimulation finished successfully.\n\n");
}

void GpuMesh::finalize() {
    if (m_pPartitioned) {
        lfm_partitioned_destroy(m_pPartitioned);   // owns the partition solvers
        m_pPartitioned = nullptr;
        for (Part& p : m_parts) p.solver = nullptr;
    }
    for (Part& p : m_parts) {
        if (p.solver) lfm_solver_destroy(p.solver);
        p.solver = nullptr;
        delete p.sc;
        p.sc = nullptr;
    }
}

}  // namespace fastmesh
