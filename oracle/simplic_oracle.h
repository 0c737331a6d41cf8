/*
 * SimPLIC CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A serial FP64 restatement of the reference SimPLIC step
 * (daidezhi/geometricVofExt, src/SimPLIC) written to check the CUDA path.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it; the product library never links, calls or falls back to it.
 *
 * Parity status: the reference cannot be compiled anywhere this project runs
 * (every SimPLIC file includes OpenFOAM v2312 headers, which are absent), so
 * the restatement's agreement with the real reference binary is not
 * verifiable bit for bit.  It is pinned where the reference holds data: the
 * golden 64^3 "exact" fields and exactInitialVol of
 * applications/test/calcVofAdvectionErrors (see tests/test_oracle_golden.py).
 * Pieces that live in OpenFOAM itself (least-squares gradient, cell-point
 * interpolation, upwind interpolation, surfaceIntegrate, face centre/area,
 * stable sortedOrder) are restated from their published methods with the
 * choices documented next to each function.
 *
 * Compiled with -ffp-contract=off so that no a*b+c is fused: every result
 * is the IEEE-754 double of the written expression order.
 */
#ifndef SIMPLIC_ORACLE_H
#define SIMPLIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_mesh {
    int32_t n_points;
    int32_t n_faces;
    int32_t n_internal_faces;
    int32_t n_cells;
    const double*  points;         /* [3*n_points]                     */
    const int32_t* face_offsets;   /* [n_faces+1]                      */
    const int32_t* face_points;    /* stored order, normal out of owner */
    const int32_t* owner;          /* [n_faces]                        */
    const int32_t* neighbour;      /* [n_internal_faces]               */
    const double*  cell_centres;   /* [3*n_cells]                      */
    const double*  cell_volumes;   /* [n_cells]                        */
    const double*  face_centres;   /* [3*n_faces]                      */
    const double*  face_areas;     /* [3*n_faces]                      */
    const double*  face_mag_areas; /* [n_faces]                        */
} oracle_mesh;

typedef struct oracle_controls {
    double  mixed_cell_tol;   /* reconstruction.C:502 */
    int32_t n_alpha_bounds;   /* advection.C:455 */
    double  snap_tol;         /* advection.C:456 */
    int32_t clip;             /* advection.C:457 */
    int32_t n_threads;        /* 1 = serial reference order; >1 OpenMP */
    int32_t orientation;      /* 0 isoAlphaGrad (LS), 1 isoRDF (reconstruction.C:60-68) */
    double  rdf_tol;          /* tol        1e-6 (reconstruction.C:513) */
    double  rdf_rel_tol;      /* relTol     0.1  (reconstruction.C:514) */
    int32_t rdf_iterations;   /* iterations 5    (reconstruction.C:515) */
    int32_t split_warped_face;/* splitWarpedFace false (reconstruction.C:506) */
} oracle_controls;

void* oracle_create(const oracle_mesh* mesh, const oracle_controls* ctrl);
void  oracle_destroy(void* h);

/* reconstruction::mapAlphaField (reconstruction.C:725-784) on this mesh:
 * cells with lower <= alpha <= upper get the volume fraction of the plane
 * (normal [3 n_cells], distance [n_cells]). */
int oracle_map_alpha_field(void* h, double* alpha, const double* normal, const double* distance, double lower,
                           double upper);

/* PLIC polygons of the last reconstruct (reconstruction.C:787-835): pass
 * NULL outputs to get the counts; offsets [n_polys + 1], pts [3 n_points],
 * cells [n_polys], ascending in cell. */
int oracle_interface_polygons(void* h, int32_t* n_polys, int32_t* n_points, int32_t* offsets, double* pts,
                              int32_t* cells);

/* the angle of (x, y) that orders the PLIC polygon points: atan2 made of
 * correctly rounded operations only (within a few ulp of the C library's) */
double oracle_plane_angle(double y, double x);

/* isoRDF iterations of the last reconstruct (0 with isoAlphaGrad) */
int32_t oracle_rdf_iterations(void* h);

/* reconstruction::reconstruct() on alpha (reconstruction.C:680-722). */
int oracle_reconstruct(void* h, const double* alpha);

/* advection::advect<Sp,Su>() (advectionTemplates.C:352-418).
 * alpha: in = current alpha (used for the upwind flux), out = new alpha.
 * alpha_old: NULL -> same as the incoming alpha.
 * U_boundary / alpha_boundary: NULL -> zero-gradient (owner value).
 * Sp / Su: NULL -> zeroField. */
int oracle_advect(void* h, double* alpha, const double* alpha_old,
                  const double* phi, const double* U, const double* U_boundary,
                  const double* alpha_boundary, double dt,
                  const double* Sp, const double* Su);

int32_t oracle_n_mixed(void* h);
void oracle_get_mixed(void* h, int32_t* cells, int32_t* status);
void oracle_get_interface(void* h, double* n, double* d, double* c, double* s);
void oracle_get_alpha_phi(void* h, double* alpha_phi);
void oracle_get_dvf(void* h, double* dvf);
void oracle_get_face_flatness(void* h, double* flat);
/* 1 for faces whose dVf came from the Simpson time integration */
void oracle_get_cut_faces(void* h, uint8_t* mask);
/* reconstruction / advection wall time (s); n_bound[0] = bounding passes
 * run, n_bound[1] = most overshooting cells treated in one pass */
void oracle_get_stats(void* h, double* times2, int32_t* n_bound);

/* unit-level entry points (for known-answer tests) */
int oracle_calc_sub_face(const double* pts, int32_t n, const double* normal,
                         double distance, double* centre, double* area);
int oracle_calc_sub_cell(void* h, int32_t cell, const double* normal,
                         double distance, double* vof, double* centre,
                         double* area);
int oracle_find_signed_distance(void* h, int32_t cell, double alpha,
                                const double* normal, double* d,
                                double* centre, double* area);
double oracle_time_integrated_face_flux(void* h, int32_t face,
                                        const double* normal, double d,
                                        double Un0, double dt, double phi,
                                        double magSf);
void oracle_interpolate_U(void* h, int32_t cell, const double* x,
                          const double* U, const double* U_boundary,
                          double* out);

#ifdef __cplusplus
}
#endif
#endif
