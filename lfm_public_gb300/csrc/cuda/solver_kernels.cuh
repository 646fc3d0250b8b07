// Device kernels of the explicit finite-volume time step (sm_103a).
//
// One RK stage of the reference (src/mesh_solver.cpp:500-672) becomes five
// kernels over structure-of-arrays data, all deterministic (no atomics on
// values, every sum in a fixed order):
//
//   k_prep     per cell and ghost: boundary-ghost state (set_boundary_conditions,
//              src/cfd_v0.cpp:1009-1221) and the primitives every face reads
//              (1/rho, u, R psi = p/rho, c), computed once per stage instead of
//              once per face side.
//   k_grad     per cell, gather over incident faces: Gauss-linear gradients of
//              rho, p and u that M2AUSM's minmod reconstruction reads
//              (calc_gradients_M2AUSM, :1383-1495). Only with M2AUSM + minmod;
//              the gradients of calc_gradients (:1500-1567) never reach the M1/M2
//              flux, so that pass is not run for them.
//   k_vis      per cell, gather: dudx, dTdx, then sigmaU from the
//              completed gradient (calc_VIS, :1743-1860). Skipped when mu = 0 and
//              the scheme does not read dudx, because every viscous face term is
//              then an exact zero.
//   k_flux     per flux face: the face rhs of one_rk_step_M1 / _M2 / _M2AUSM
//              (:2529-2796, :1896-2133, :2185-2489) into a face buffer.
//   k_update   per cell, gather of the face rhs in ascending face order (the
//              reference's scatter order), sponge source and the low-storage RK
//              update (:2800-2822).
//
// The gather replaces the reference's scatter: within a stage every face is
// evaluated once from the stage-start state, because a cell's owned faces
// always point to cells the reference updates later, so the sequential
// scatter-and-update is a Jacobi stage. Geometry is seen from the reference's
// processing side P of each face.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lfm {
namespace dev {

constexpr int kSchemeM1 = 0;
constexpr int kSchemeM2 = 1;
constexpr int kSchemeAUSM = 2;

// Free-stream reference state of the FP32-bulk perturbation form, rounded
// to FP32 from FP64 values computed on the host.
struct RefState32 {
    float rho, U[3], m[3];    // rho_inf, U_inf, rho_inf U_inf
    float Rpsi, p, H, gh;     // p/rho, p, total enthalpy, gamma / (gamma - 1)
    float gamma, gm1, Rinv, mu, kcond;   // gas constants (FP32 copies)
};

// Arguments shared by the kernels (all device pointers).
// Fixed-width cell -> face table (Args::cfEll): four entries per 2D cell
// (quads, triangles), six per 3D cell (hexahedra, prisms, tetrahedra).
template <int D>
constexpr int kEllWidth = D == 2 ? 4 : 6;
constexpr int kEllPad = -2147483647 - 1;

template <typename T>
struct Args {
    int D, nq;
    int nc, ng, nf, nt;       // cells, ghosts, flux faces, cells + ghosts + halos
    int nh;                   // processor-face halos (after the ghosts; filled by copies)
    // state (FP64 RK registers)
    double* q;                // nq x nt
    T* dq;                    // nq x nc RK register: FP64, or FP32 in the FP32-bulk form
                              // (it holds one step's increments and restarts every step)
    // per cell + ghost, computed every stage
    T* prim;                  // FP64: (D + 3) x nt: 1/rho, u[D], R psi, c
                              // FP32: (2D + 3) x nt: rho', m'[D], u'[D], R psi', c
    T* primW;                 // where an update writes the next stage's primitives: prim, or
                              // (fused flux-update stages) the other of two buffers, which no
                              // thread of that launch reads
    T* V;                     // (D^2 + 2D) x nt: dudx, dTdx, sigmaU
    T* grad;                  // (2D + D^2) x nt: rho_grad, p_grad, U_grad (M2AUSM)
    T* flux;                  // nq x nf face rhs
    double* res;              // nq x nc stage-0 residual per cell (or null)
    // faces
    const int* fP;
    const int* fN;
    const uint8_t* fGhost;
    const T* S;               // D x nf
    const T* d;               // D x nf
    const T* w;
    const T* smag;
    const T* dinv;            // 1/|d|
    const T* dnorm;           // D x nf
    const T* dmag;            // |delta|
    const T* K;               // D x nf
    const T* lapc;            // |delta| / |d| per face
    const T* wN;              // FP64 path: 1 - w per face (the linear weight of N)
    // cells
    const double* volInv;
    const float* volInv32;    // FP32 copy (FP32-bulk gradient kernels)
    const T* sponge;          // sponge coefficient sigma per cell
    const int* cfOff;         // nc + 1
    const int* cfList;        // face index, negative (~f) when the cell is N
    const int* cfNbr;         // per cfList entry: the cell (or ghost, halo) across the face
    const T* cfSoN;           // FP64 path: (cfList entries) x D, the linear weight of the cell
                              // across the entry's face times S / V seen from the entry's cell
    const T* cellSoW;         // FP64 path: nc x D, the sum over the cell's faces of its own
                              // linear weight times S / V (Gauss gradient of cell c:
                              // v_c cellSoW_c + sum over entries of v_across cfSoN)
    const T* smagC;           // Smagorinsky LES: the constant each cell's tauMC is built with
                              // (V then holds D x D more rows: its SGS stress), or null
    const uint8_t* cellGhosts;  // FP32-bulk single case: boundary faces of each cell
                                // (its update writes their ghosts' primitives), or null
    const int* fOwn;          // FP32-bulk cell-centred flux: nc + 1 offsets, the flux faces that
                              // cell c owns (is P of) are fOwn[c] .. fOwn[c + 1] - 1 (the faces
                              // are stored by owner); null where the face-per-thread kernel runs
    const int* cfEll;         // FP32-bulk update gather (single cases beyond L2, batch cases):
                              // the cfList entries of each cell at a fixed width
                              // (kEllWidth<D>), entry k of cell c at k * nc + c, kEllPad
                              // after the cell's faces; null where unused or a cell has more
                              // faces (the update then gathers through cfOff / cfList)
    // ghosts
    const int* gCell;
    const int* gKind;
    const int* gFace;
    // constants
    double gamma, gm1, Rinv, rhoInf, EInf, pInf, TInf, UInf[3], mu, kcond;
    double gh;                // gamma / (gamma - 1): enthalpy per unit R psi
    double mu23;              // 2/3 mu (the trace term of the deviatoric stress)
    // FP32-bulk: conservative reference state q_ref = (rho_inf, rho_inf U_inf,
    // rho_inf E_inf) in FP64 (index = variable) and its derived FP32 constants
    double qRef[5];
    double pRef;              // (gamma - 1)(rho_inf E_inf - rho_inf |U_inf|^2 / 2)
    RefState32 ref;
    // FP64 path: the primitives include the sound speed (read by M2AUSM only)
    int primC;
    // error flag (non-finite state)
    int* flag;
};

}  // namespace dev
}  // namespace lfm
