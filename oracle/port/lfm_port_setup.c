/* Oracle-side case set-up: from an in-memory polyMesh, the case parameters
 * and the initial fields to the flattened solver description (lfm_solver_desc)
 * that the oracle port advances.
 *
 * TEST INFRASTRUCTURE ONLY, like lfm_port.c: tests, the smoke check and the
 * CPU legs of bench.py use it so that the oracle needs nothing from the
 * device library. It is an independent restatement, in plain C, of the steps
 * the reference takes between reading a polyMesh and its first stage:
 *
 *   OpenFOAM (third party, "v2112 or higher", reference README.md:30; not in
 *   the reference tree) -- the published primitiveMesh construction:
 *     cell face lists: every face appended to its owner's list in face
 *       order, then every internal face to its neighbour's list;
 *     face centre and area: triangles are exact, larger faces a fan of
 *       triangles about the point average, centre area-weighted;
 *     cell centre and volume: pyramids from every face to the average of the
 *       cell's face centres, centre volume-weighted.
 *   polyMeshReaderOF/polyMeshReaderOF.cpp:47-64   faces of 'empty' patches
 *                                                 are invalid
 *   polyMeshReaderOF/polyMeshReaderOF.cpp:230-248 cyclic partner face
 *   polyMeshReaderOF/polyMeshReaderOF.cpp:501-552 submesh split: cells that
 *                                                 touch a point of a
 *                                                 non-empty patch -> 0
 *   src/mesh_reader.cpp:263-460     face area normals; neighbour-centre
 *                                   vectors (cyclic translated, boundary
 *                                   ghosts mirrored)
 *   src/cfd_v0.cpp:759-861          S, d, linear weight, 1/V per cell-face
 *   src/cfd_v0.cpp:277-339          reorder_faces: a face belongs to the
 *                                   side with the smaller (submesh, index)
 *   src/cfd_v0.cpp:344-420          one boundary ghost per boundary face
 *   src/cfd_v0.cpp:972-1005         patch -> boundary-condition kind
 *   src/cfd_v0.cpp:866-967          free stream, sponge, initial state
 *   src/cfd_v0.cpp:1573-1737        Smagorinsky constant (line 1601)
 *   src/cfd_v0.cpp:86-128           low-storage RK coefficients
 *   src/cfd_v0.cpp:2687-2766        the per-face constants |S|, 1/|d|, d/|d|,
 *                                   |delta|, K = S - delta, evaluated once
 *
 * Whole cases only (no processor patches) in the reference's own cell order
 * (no renumbering). Every expression is evaluated in the reference's order;
 * build with -ffp-contract=off. */
#include "lfm_port.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct lfm_port_case {
    int dim, nq, solver, rk_order, minmod, residuals;
    int64_t nc, nc0, ng, nf;
    int64_t *face_p, *face_n;
    uint8_t* face_ghost;
    double *S, *d, *w, *smag, *dmag_inv, *dnorm, *delta_mag, *K;
    double *vol_inv, *sponge, *smag_c, *q0;
    int64_t* ghost_cell;
    int* ghost_kind;
    int32_t* ghost_patch;
    int64_t *cf_off, *cf_list;
    int8_t* cf_sign;
    int64_t* cs_off;
    double* cs;
    int64_t* cell_id;   /* polyMesh cell of each solver-order cell */
    double gamma, Rgas, rhoInf, EInf, pInf, TInf, UInf[3], mu, Cp, PrInv;
    double rkA[8], rkB[8];
};

static char g_err[256];

const char* lfm_port_last_error(void) { return g_err; }

static int fail(const char* msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return -1;
}

static void* zalloc(int64_t n, size_t sz) { return calloc((size_t)(n > 0 ? n : 1), sz); }

/* ---- OpenFOAM geometry ------------------------------------------------- */
typedef struct {
    int64_t nf, ni, nc, np;
    const double* pts;
    const int64_t *fo, *fp, *own, *nei;
    int64_t *c_off, *c_faces;        /* cell -> faces, OpenFOAM's order */
    double *fA, *fC, *cC, *cV;       /* [3] per face / cell, volumes */
} Geom;

static void face_geometry(Geom* g) {
    for (int64_t f = 0; f < g->nf; ++f) {
        const int64_t* fp = g->fp + g->fo[f];
        const int64_t np = g->fo[f + 1] - g->fo[f];
        double* ctr = g->fC + 3 * f;
        double* area = g->fA + 3 * f;
        if (np == 3) {
            const double *a = g->pts + 3 * fp[0], *b = g->pts + 3 * fp[1], *c = g->pts + 3 * fp[2];
            double u[3], v[3];
            for (int k = 0; k < 3; ++k) {
                ctr[k] = (1.0 / 3.0) * (a[k] + b[k] + c[k]);
                u[k] = b[k] - a[k];
                v[k] = c[k] - a[k];
            }
            area[0] = 0.5 * (u[1] * v[2] - u[2] * v[1]);
            area[1] = 0.5 * (u[2] * v[0] - u[0] * v[2]);
            area[2] = 0.5 * (u[0] * v[1] - u[1] * v[0]);
            continue;
        }
        double avg[3];
        for (int k = 0; k < 3; ++k) avg[k] = g->pts[3 * fp[0] + k];
        for (int64_t i = 1; i < np; ++i)
            for (int k = 0; k < 3; ++k) avg[k] += g->pts[3 * fp[i] + k];
        for (int k = 0; k < 3; ++k) avg[k] /= (double)np;
        double sn[3] = {0, 0, 0}, sac[3] = {0, 0, 0}, sa = 0.0;
        for (int64_t i = 0; i < np; ++i) {
            const double* p0 = g->pts + 3 * fp[i];
            const double* p1 = g->pts + 3 * fp[i + 1 == np ? 0 : i + 1];
            double c[3], u[3], v[3], n[3];
            for (int k = 0; k < 3; ++k) {
                c[k] = p0[k] + p1[k] + avg[k];
                u[k] = p1[k] - p0[k];
                v[k] = avg[k] - p0[k];
            }
            n[0] = u[1] * v[2] - u[2] * v[1];
            n[1] = u[2] * v[0] - u[0] * v[2];
            n[2] = u[0] * v[1] - u[1] * v[0];
            const double a = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; ++k) {
                sn[k] += n[k];
                sac[k] += a * c[k];
            }
            sa += a;
        }
        for (int k = 0; k < 3; ++k) {
            if (sa < 1.0e-150) {
                ctr[k] = avg[k];
                area[k] = 0.0;
            } else {
                ctr[k] = (1.0 / 3.0) * sac[k] / sa;
                area[k] = 0.5 * sn[k];
            }
        }
    }
}

static void pyramid(Geom* g, const double* est, int64_t f, int64_t c, int is_owner) {
    const double *fc = g->fC + 3 * f, *fa = g->fA + 3 * f, *ce = est + 3 * c;
    double pyr3;
    if (is_owner)
        pyr3 = fa[0] * (fc[0] - ce[0]) + fa[1] * (fc[1] - ce[1]) + fa[2] * (fc[2] - ce[2]);
    else
        pyr3 = fa[0] * (ce[0] - fc[0]) + fa[1] * (ce[1] - fc[1]) + fa[2] * (ce[2] - fc[2]);
    for (int k = 0; k < 3; ++k) g->cC[3 * c + k] += pyr3 * ((3.0 / 4.0) * fc[k] + (1.0 / 4.0) * ce[k]);
    g->cV[c] += pyr3;
}

static void cell_geometry(Geom* g) {
    double* est = zalloc(3 * g->nc, sizeof(double));
    int64_t* nface = zalloc(g->nc, sizeof(int64_t));
    for (int64_t f = 0; f < g->nf; ++f) {
        for (int k = 0; k < 3; ++k) est[3 * g->own[f] + k] += g->fC[3 * f + k];
        ++nface[g->own[f]];
    }
    for (int64_t f = 0; f < g->ni; ++f) {
        for (int k = 0; k < 3; ++k) est[3 * g->nei[f] + k] += g->fC[3 * f + k];
        ++nface[g->nei[f]];
    }
    for (int64_t c = 0; c < g->nc; ++c)
        for (int k = 0; k < 3; ++k) est[3 * c + k] /= (double)nface[c];
    for (int64_t f = 0; f < g->nf; ++f) pyramid(g, est, f, g->own[f], 1);
    for (int64_t f = 0; f < g->ni; ++f) pyramid(g, est, f, g->nei[f], 0);
    for (int64_t c = 0; c < g->nc; ++c) {
        for (int k = 0; k < 3; ++k) {
            if (fabs(g->cV[c]) > 1.0e-300)
                g->cC[3 * c + k] /= g->cV[c];
            else
                g->cC[3 * c + k] = est[3 * c + k];
        }
        g->cV[c] *= (1.0 / 3.0);
    }
    free(est);
    free(nface);
}

static int cell_faces(Geom* g) {
    g->c_off = zalloc(g->nc + 1, sizeof(int64_t));
    for (int64_t f = 0; f < g->nf; ++f) ++g->c_off[g->own[f] + 1];
    for (int64_t f = 0; f < g->ni; ++f) ++g->c_off[g->nei[f] + 1];
    for (int64_t c = 0; c < g->nc; ++c) g->c_off[c + 1] += g->c_off[c];
    g->c_faces = zalloc(g->c_off[g->nc], sizeof(int64_t));
    int64_t* fill = zalloc(g->nc, sizeof(int64_t));
    for (int64_t c = 0; c < g->nc; ++c) fill[c] = g->c_off[c];
    for (int64_t f = 0; f < g->nf; ++f) g->c_faces[fill[g->own[f]]++] = f;
    for (int64_t f = 0; f < g->ni; ++f) g->c_faces[fill[g->nei[f]]++] = f;
    free(fill);
    return 0;
}

/* ---- reader queries ---------------------------------------------------- */
typedef struct {
    const lfm_polymesh* m;
    Geom* g;
    int* patch_of;       /* face -> patch or -1 */
    int64_t* cyc_shift;  /* patch -> partner start - own start (cyclic), or 0 */
    int* cyclic;         /* patch is a coupled cyclic */
    uint8_t* valid;      /* face not on an 'empty' patch */
} Reader;

static int64_t cyclic_face(const Reader* r, int64_t f) {
    const int b = r->patch_of[f];
    if (b < 0 || !r->cyclic[b]) return f;
    return f + r->cyc_shift[b];
}

static int64_t face_neighbour(const Reader* r, int64_t f) {
    if (f < r->g->ni) return r->g->nei[f];
    const int64_t c = cyclic_face(r, f);
    return c == f ? -1 : r->g->own[c];
}

typedef struct {
    int64_t face;
    int type;          /* 0 cell, 1 boundary ghost */
    int64_t nb;        /* solver index of the neighbour cell */
    int nb_sm;
    int64_t nb_local;
    int bound;
    double S[3], d[3], w;
    int owned;
} Slot;

static void rk_coefficients(int order, double* A, double* B) {
    static const double A4[4] = {0.0, -756391.0 / 934407.0, -36441873.0 / 15625000.0, -1953125.0 / 1085297.0};
    static const double B4[4] = {8.0 / 141.0, 6627.0 / 2000.0, 609375.0 / 1085297.0, 198961.0 / 526383.0};
    static const double A5[5] = {0.0, -0.4178904745, -1.192151694643, -1.697784692471, -1.514183444257};
    static const double B5[5] = {0.1496590219993, 0.3792103129999, 0.8229550293869, 0.6994504559488,
                                 0.1530572479681};
    memset(A, 0, 8 * sizeof(double));
    memset(B, 0, 8 * sizeof(double));
    if (order <= 1) {
        A[0] = 0.0;
        B[0] = 1.0;
    } else if (order == 2) {
        A[1] = -1.0;
        B[0] = 1.0;
        B[1] = 0.5;
    } else if (order <= 4) {
        memcpy(A, A4, sizeof A4);
        memcpy(B, B4, sizeof B4);
    } else {
        memcpy(A, A5, sizeof A5);
        memcpy(B, B5, sizeof B5);
    }
}

static int ghost_kind_of(const char* type, const char* name) {
    if (strcmp(type, "wall") == 0) return LFM_GHOST_WALL;
    if (strcmp(type, "farfield") == 0) return LFM_GHOST_FARFIELD;
    if (strcmp(type, "patch") == 0) {
        if (!strcmp(name, "inlet") || !strcmp(name, "Inlet") || !strcmp(name, "Inflow") || !strcmp(name, "inflow"))
            return LFM_GHOST_INLET;
        if (!strcmp(name, "outlet") || !strcmp(name, "Outlet") || !strcmp(name, "Outflow") ||
            !strcmp(name, "outflow"))
            return LFM_GHOST_OUTLET;
    }
    return LFM_GHOST_NONE;
}

void lfm_port_case_free(lfm_port_case* c) {
    if (!c) return;
    void* arrays[] = {c->face_p, c->face_n, c->face_ghost, c->S, c->d, c->w, c->smag, c->dmag_inv, c->dnorm,
                      c->delta_mag, c->K, c->vol_inv, c->sponge, c->smag_c, c->q0, c->ghost_cell, c->ghost_kind,
                      c->ghost_patch, c->cf_off, c->cf_list, c->cf_sign, c->cs_off, c->cs, c->cell_id};
    for (size_t i = 0; i < sizeof arrays / sizeof arrays[0]; ++i) free(arrays[i]);
    free(c);
}

static void free_geom(Geom* g) {
    free(g->c_off);
    free(g->c_faces);
    free(g->fA);
    free(g->fC);
    free(g->cC);
    free(g->cV);
}

int lfm_port_case_build(const lfm_polymesh* m, const lfm_params* prm, const lfm_fields* fld, lfm_port_case** out) {
    if (!m || !prm || !fld || !out) return fail("null argument");
    *out = NULL;
    const int D = prm->dimension;
    if (D != 2 && D != 3) return fail("dimension must be 2 or 3");
    if (prm->solver < 0 || prm->solver > 2 || prm->rk_order < 0 || prm->rk_order > 5) return fail("bad parameters");
    if (prm->renumber != LFM_RENUMBER_NONE) return fail("the oracle runs the reference's own cell order only");
    if (m->n_cells <= 0 || m->n_faces <= 0 || !fld->p || !fld->T || !fld->U || (prm->Ls > 0 && !fld->alpha))
        return fail("incomplete case");
    for (int b = 0; b < m->n_patches; ++b)
        if (!strncmp(m->patch_type[b], "processor", 9)) return fail("processor patches: whole cases only");

    Geom g;
    memset(&g, 0, sizeof g);
    g.nf = m->n_faces;
    g.ni = m->n_internal_faces;
    g.nc = m->n_cells;
    g.np = m->n_points;
    g.pts = m->points;
    g.fo = m->face_offsets;
    g.fp = m->face_points;
    g.own = m->owner;
    g.nei = m->neighbour;
    for (int64_t f = 0; f < g.nf; ++f)
        if (g.own[f] < 0 || g.own[f] >= g.nc) return fail("owner label out of range");
    for (int64_t f = 0; f < g.ni; ++f)
        if (g.nei[f] < 0 || g.nei[f] >= g.nc) return fail("neighbour label out of range");
    g.fA = zalloc(3 * g.nf, sizeof(double));
    g.fC = zalloc(3 * g.nf, sizeof(double));
    g.cC = zalloc(3 * g.nc, sizeof(double));
    g.cV = zalloc(g.nc, sizeof(double));
    cell_faces(&g);
    face_geometry(&g);
    cell_geometry(&g);

    Reader r;
    r.m = m;
    r.g = &g;
    r.patch_of = zalloc(g.nf, sizeof(int));
    r.valid = zalloc(g.nf, 1);
    r.cyclic = zalloc(m->n_patches, sizeof(int));
    r.cyc_shift = zalloc(m->n_patches, sizeof(int64_t));
    for (int64_t f = 0; f < g.nf; ++f) {
        r.patch_of[f] = -1;
        r.valid[f] = 1;
    }
    for (int b = 0; b < m->n_patches; ++b) {
        for (int64_t f = m->patch_start[b]; f < m->patch_start[b] + m->patch_size[b]; ++f) {
            if (r.patch_of[f] < 0) r.patch_of[f] = b;   /* the first patch holding the face */
            if (!strcmp(m->patch_type[b], "empty")) r.valid[f] = 0;
        }
        if (!strcmp(m->patch_type[b], "cyclic") && m->patch_neighbour && m->patch_neighbour[b])
            for (int q = 0; q < m->n_patches; ++q)
                if (!strcmp(m->patch_name[q], m->patch_neighbour[b])) {
                    r.cyclic[b] = 1;
                    r.cyc_shift[b] = m->patch_start[q] - m->patch_start[b];
                    break;
                }
    }
    for (int64_t f = 0; f < g.ni; ++f) r.patch_of[f] = -1;

    /* submesh split */
    int* sm = zalloc(g.nc, sizeof(int));
    if (m->cell_submesh) {
        for (int64_t c = 0; c < g.nc; ++c) sm[c] = (int)m->cell_submesh[c];
    } else {
        uint8_t* bpt = zalloc(g.np, 1);
        for (int b = 0; b < m->n_patches; ++b) {
            if (!strcmp(m->patch_type[b], "empty")) continue;
            for (int64_t f = m->patch_start[b]; f < m->patch_start[b] + m->patch_size[b]; ++f)
                for (int64_t k = g.fo[f]; k < g.fo[f + 1]; ++k) bpt[g.fp[k]] = 1;
        }
        for (int64_t c = 0; c < g.nc; ++c) {
            int interior = 1;
            for (int64_t i = g.c_off[c]; i < g.c_off[c + 1] && interior; ++i) {
                const int64_t f = g.c_faces[i];
                for (int64_t k = g.fo[f]; k < g.fo[f + 1] && interior; ++k) interior = !bpt[g.fp[k]];
            }
            sm[c] = interior ? 1 : 0;
        }
        free(bpt);
    }
    int nsub = 0;
    for (int64_t c = 0; c < g.nc; ++c)
        if (sm[c] + 1 > nsub) nsub = sm[c] + 1;

    lfm_port_case* pc = calloc(1, sizeof *pc);
    pc->dim = D;
    pc->nq = D + 2;
    pc->nc = g.nc;
    /* solver order: submesh 0 cells ascending, then submesh 1, ... */
    int64_t* cell_of = zalloc(g.nc, sizeof(int64_t));   /* solver index -> polyMesh cell */
    int64_t* solver_of = zalloc(g.nc, sizeof(int64_t));
    int64_t* local_of = zalloc(g.nc, sizeof(int64_t));
    int64_t k = 0;
    for (int s = 0; s < nsub; ++s) {
        int64_t loc = 0;
        for (int64_t c = 0; c < g.nc; ++c)
            if (sm[c] == s) {
                cell_of[k] = c;
                solver_of[c] = k++;
                local_of[c] = loc++;
            }
        if (s == 0) pc->nc0 = k;
    }

    /* per cell-face slots */
    int64_t* slot_off = zalloc(g.nc + 1, sizeof(int64_t));
    for (int64_t ci = 0; ci < g.nc; ++ci) {
        const int64_t cell = cell_of[ci];
        int64_t nv = 0;
        for (int64_t i = g.c_off[cell]; i < g.c_off[cell + 1]; ++i) nv += r.valid[g.c_faces[i]];
        slot_off[ci + 1] = slot_off[ci] + nv;
    }
    Slot* slots = zalloc(slot_off[g.nc], sizeof(Slot));
    int err = 0;
    for (int64_t ci = 0; ci < g.nc && !err; ++ci) {
        const int64_t cell = cell_of[ci];
        const double* xc = g.cC + 3 * cell;
        Slot* sl = slots + slot_off[ci];
        for (int64_t i = g.c_off[cell]; i < g.c_off[cell + 1]; ++i) {
            const int64_t f = g.c_faces[i];
            if (!r.valid[f]) continue;
            const int64_t own = g.own[f], nbr = face_neighbour(&r, f);
            const int64_t other = own == cell ? nbr : own;
            sl->face = f;
            sl->bound = r.patch_of[f];
            if (other != -1) {
                sl->type = 0;
                sl->nb = solver_of[other];
                sl->nb_sm = sm[other];
                sl->nb_local = local_of[other];
            } else {
                sl->type = 1;
                if (sm[cell] != 0) err = 1;   /* the reference has no ghost for submesh 1 (src/cfd_v0.cpp:352-353) */
            }
            const double sign = own == cell ? 1.0 : -1.0;
            const double* xf = g.fC + 3 * f;
            double dP[3], dN[3];
            for (int dd = 0; dd < D; ++dd) {
                sl->S[dd] = sign * g.fA[3 * f + dd];
                dP[dd] = xc[dd] - xf[dd];
            }
            if (sl->type == 1) {
                double s2 = 0.0, dps = 0.0;
                for (int dd = 0; dd < D; ++dd) s2 += sl->S[dd] * sl->S[dd];
                for (int dd = 0; dd < D; ++dd) dps += dP[dd] * sl->S[dd];
                for (int dd = 0; dd < D; ++dd) sl->d[dd] = 2.0 * fabs(dps) * sl->S[dd] / s2;
            } else {
                const double *xo = g.cC + 3 * own, *xn = g.cC + 3 * nbr;
                double vn[3];
                for (int dd = 0; dd < D; ++dd) vn[dd] = xn[dd] - xo[dd];
                const int64_t cyc = cyclic_face(&r, f);
                if (cyc != f)
                    for (int dd = 0; dd < D; ++dd) vn[dd] += g.fC[3 * f + dd] - g.fC[3 * cyc + dd];
                for (int dd = 0; dd < D; ++dd) sl->d[dd] = sign * vn[dd];
            }
            for (int dd = 0; dd < D; ++dd) dN[dd] = dP[dd] + sl->d[dd];
            double wn = 0.0, wd = 0.0;
            for (int dd = 0; dd < D; ++dd) {
                wn += sl->S[dd] * dN[dd];
                wd += (-sl->S[dd] * dP[dd] + sl->S[dd] * dN[dd]);
            }
            sl->w = wn / wd;
            if (sl->type != 0)
                sl->owned = 1;
            else
                sl->owned = !(sl->nb_sm < sm[cell] || (sl->nb_sm == sm[cell] && sl->nb_local < local_of[cell]));
            ++sl;
        }
    }
    if (err) {
        free(slots), free(slot_off), free(cell_of), free(solver_of), free(local_of), free(sm);
        free(r.patch_of), free(r.valid), free(r.cyclic), free(r.cyc_shift);
        free_geom(&g);
        lfm_port_case_free(pc);
        return fail("a boundary face belongs to an interior-submesh cell");
    }

    /* flux faces in processing order, ghosts, per-face constants */
    int64_t nf = 0, ng = 0;
    for (int64_t e = 0; e < slot_off[g.nc]; ++e) {
        nf += slots[e].owned;
        ng += slots[e].owned && slots[e].type == 1;
    }
    pc->nf = nf;
    pc->ng = ng;
    pc->face_p = zalloc(nf, sizeof(int64_t));
    pc->face_n = zalloc(nf, sizeof(int64_t));
    pc->face_ghost = zalloc(nf, 1);
    pc->S = zalloc(D * nf, sizeof(double));
    pc->d = zalloc(D * nf, sizeof(double));
    pc->w = zalloc(nf, sizeof(double));
    pc->smag = zalloc(nf, sizeof(double));
    pc->dmag_inv = zalloc(nf, sizeof(double));
    pc->dnorm = zalloc(D * nf, sizeof(double));
    pc->delta_mag = zalloc(nf, sizeof(double));
    pc->K = zalloc(D * nf, sizeof(double));
    pc->ghost_cell = zalloc(ng, sizeof(int64_t));
    pc->ghost_kind = zalloc(ng, sizeof(int));
    pc->ghost_patch = zalloc(ng, sizeof(int32_t));
    int64_t fi = 0, gi = 0;
    for (int64_t ci = 0; ci < g.nc; ++ci) {
        for (int64_t e = slot_off[ci]; e < slot_off[ci + 1]; ++e) {
            const Slot* sl = slots + e;
            if (!sl->owned) continue;
            pc->face_p[fi] = ci;
            if (sl->type == 1) {
                pc->ghost_cell[gi] = ci;
                pc->ghost_kind[gi] = ghost_kind_of(m->patch_type[sl->bound], m->patch_name[sl->bound]);
                pc->ghost_patch[gi] = sl->bound;
                pc->face_n[fi] = g.nc + gi;
                pc->face_ghost[fi] = 1;
                ++gi;
            } else {
                pc->face_n[fi] = sl->nb;
            }
            for (int dd = 0; dd < D; ++dd) {
                pc->S[dd * nf + fi] = sl->S[dd];
                pc->d[dd * nf + fi] = sl->d[dd];
            }
            pc->w[fi] = sl->w;
            double dm = sl->d[0] * sl->d[0];
            for (int dd = 1; dd < D; ++dd) dm += sl->d[dd] * sl->d[dd];
            dm = sqrt(dm);
            const double dinv = 1.0 / dm;
            double sm2 = 0.0;
            for (int dd = 0; dd < D; ++dd) sm2 += sl->S[dd] * sl->S[dd];
            const double smag = sqrt(sm2);
            double sd = sl->S[0] * sl->d[0];
            for (int dd = 1; dd < D; ++dd) sd += sl->S[dd] * sl->d[dd];
            double dl = 0.0;
            for (int dd = 0; dd < D; ++dd) {
                const double delta = sl->d[dd] * smag * smag / sd;
                dl += delta * delta;
                pc->K[dd * nf + fi] = sl->S[dd] - delta;
                pc->dnorm[dd * nf + fi] = sl->d[dd] * dinv;
            }
            pc->smag[fi] = smag;
            pc->dmag_inv[fi] = dinv;
            pc->delta_mag[fi] = sqrt(dl);
            ++fi;
        }
    }

    /* cell -> face incidence in ascending face order */
    pc->cf_off = zalloc(g.nc + 1, sizeof(int64_t));
    for (int64_t f = 0; f < nf; ++f) {
        ++pc->cf_off[pc->face_p[f] + 1];
        if (pc->face_n[f] < g.nc) ++pc->cf_off[pc->face_n[f] + 1];
    }
    for (int64_t c = 0; c < g.nc; ++c) pc->cf_off[c + 1] += pc->cf_off[c];
    pc->cf_list = zalloc(pc->cf_off[g.nc], sizeof(int64_t));
    pc->cf_sign = zalloc(pc->cf_off[g.nc], 1);
    int64_t* fill = zalloc(g.nc, sizeof(int64_t));
    for (int64_t c = 0; c < g.nc; ++c) fill[c] = pc->cf_off[c];
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t p = pc->face_p[f], n = pc->face_n[f];
        pc->cf_list[fill[p]] = f;
        pc->cf_sign[fill[p]++] = 1;
        if (n < g.nc) {
            pc->cf_list[fill[n]] = f;
            pc->cf_sign[fill[n]++] = -1;
        }
    }
    free(fill);

    /* S of every valid face of a cell seen from it: owned slots in slot
     * order, then the others in reverse (the reordered slot order) */
    pc->cs_off = zalloc(g.nc + 1, sizeof(int64_t));
    for (int64_t c = 0; c < g.nc; ++c) pc->cs_off[c + 1] = slot_off[c + 1];
    pc->cs = zalloc(slot_off[g.nc] * D, sizeof(double));
    for (int64_t c = 0; c < g.nc; ++c) {
        int64_t o = pc->cs_off[c];
        for (int64_t e = slot_off[c]; e < slot_off[c + 1]; ++e)
            if (slots[e].owned) {
                for (int dd = 0; dd < D; ++dd) pc->cs[o * D + dd] = slots[e].S[dd];
                ++o;
            }
        for (int64_t e = slot_off[c + 1]; e-- > slot_off[c];)
            if (!slots[e].owned) {
                for (int dd = 0; dd < D; ++dd) pc->cs[o * D + dd] = slots[e].S[dd];
                ++o;
            }
    }

    /* constants and initial state */
    pc->solver = prm->solver;
    pc->rk_order = prm->rk_order;
    pc->minmod = prm->minmod != 0;
    pc->residuals = prm->residuals != 0;
    rk_coefficients(prm->rk_order, pc->rkA, pc->rkB);
    pc->pInf = prm->p_inf;
    pc->TInf = prm->T_inf;
    for (int dd = 0; dd < 3; ++dd) pc->UInf[dd] = dd < D ? prm->U_inf[dd] : 0.0;
    pc->mu = prm->mu;
    pc->Cp = prm->Cp;
    pc->Rgas = 8.31447 / prm->mol_weight * 1000;
    const double Cv = prm->Cp - pc->Rgas;
    pc->gamma = prm->Cp / Cv;
    pc->rhoInf = prm->p_inf / (pc->Rgas * prm->T_inf);
    const double gm1 = pc->gamma - 1.0;
    double u2 = 0;
    for (int dd = 0; dd < D; ++dd) u2 += pc->UInf[dd] * pc->UInf[dd];
    pc->EInf = prm->p_inf / (pc->rhoInf * gm1) + 0.5 * u2;
    pc->PrInv = 1.0 / prm->Pr;

    pc->vol_inv = zalloc(g.nc, sizeof(double));
    pc->sponge = zalloc(g.nc, sizeof(double));
    for (int64_t c = 0; c < g.nc; ++c) pc->vol_inv[c] = 1.0 / g.cV[cell_of[c]];
    if (!prm->laminar) {
        pc->smag_c = zalloc(g.nc, sizeof(double));
        for (int64_t c = 0; c < g.nc; ++c)
            pc->smag_c[c] = -(double)2.0 * pow((double)0.16 * pow(1.0 / pc->vol_inv[c], 1. / 3.), 2);
    }
    if (prm->Ls > 0) {
        const double sigma0 = 3.0 * (1.0 - prm->mach * prm->mach) / (prm->k_sponge * prm->Ls);
        for (int64_t c = 0; c < g.nc; ++c) {
            const double dist = fld->alpha[cell_of[c]];
            if (dist < prm->Ls) {
                const double x = (prm->Ls - dist) / prm->Ls;
                pc->sponge[c] = sigma0 * (x * x);
            }
        }
    }
    pc->q0 = zalloc(pc->nq * g.nc, sizeof(double));
    for (int64_t c = 0; c < g.nc; ++c) {
        const int64_t cell = cell_of[c];
        const double* U = fld->U + 3 * cell;
        const double p = fld->p[cell], T = fld->T[cell];
        double um2 = 0;
        for (int dd = 0; dd < D; ++dd) um2 += U[dd] * U[dd];
        const double rho = p / (pc->Rgas * T);
        const double E = p / (rho * gm1) + 0.5 * um2;
        pc->q0[c] = rho;
        for (int dd = 0; dd < D; ++dd) pc->q0[(dd + 1) * g.nc + c] = rho * U[dd];
        pc->q0[(D + 1) * g.nc + c] = rho * E;
    }

    pc->cell_id = cell_of;
    free(slots), free(slot_off), free(solver_of), free(local_of), free(sm);
    free(r.patch_of), free(r.valid), free(r.cyclic), free(r.cyc_shift);
    free_geom(&g);
    *out = pc;
    return 0;
}

int lfm_port_case_cell_ids(const lfm_port_case* c, int64_t* out) {
    if (!c || !out) return fail("null argument");
    memcpy(out, c->cell_id, (size_t)c->nc * sizeof(int64_t));
    return 0;
}

int lfm_port_case_describe(const lfm_port_case* c, lfm_solver_desc* d) {
    if (!c || !d) return fail("null argument");
    memset(d, 0, sizeof *d);
    d->dim = c->dim;
    d->nq = c->nq;
    d->solver = c->solver;
    d->rk_order = c->rk_order;
    d->minmod = c->minmod;
    d->residuals = c->residuals;
    d->n_cells = c->nc;
    d->n_cells0 = c->nc0;
    d->n_ghosts = c->ng;
    d->n_faces = c->nf;
    d->face_p = c->face_p;
    d->face_n = c->face_n;
    d->face_ghost = c->face_ghost;
    d->S = c->S;
    d->d = c->d;
    d->w = c->w;
    d->smag = c->smag;
    d->dmag_inv = c->dmag_inv;
    d->dnorm = c->dnorm;
    d->delta_mag = c->delta_mag;
    d->K = c->K;
    d->vol_inv = c->vol_inv;
    d->sponge = c->sponge;
    d->ghost_cell = c->ghost_cell;
    d->ghost_kind = c->ghost_kind;
    d->cell_face_offsets = c->cf_off;
    d->cell_faces = c->cf_list;
    d->cell_face_sign = c->cf_sign;
    d->cell_s_offsets = c->cs_off;
    d->cell_s = c->cs;
    d->q0 = c->q0;
    d->gamma = c->gamma;
    d->Rgas = c->Rgas;
    d->rhoInf = c->rhoInf;
    d->EInf = c->EInf;
    d->pInf = c->pInf;
    d->TInf = c->TInf;
    for (int k = 0; k < 3; ++k) d->UInf[k] = c->UInf[k];
    d->mu = c->mu;
    d->Cp = c->Cp;
    d->PrInv = c->PrInv;
    d->rkA = c->rkA;
    d->rkB = c->rkB;
    d->ghost_patch = c->ghost_patch;
    d->smag_c = c->smag_c;
    return 0;
}
