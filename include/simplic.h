/*
 * simplic.h -- C ABI of the GB300 SimPLIC volume-fraction advection step.
 *
 * One handle replaces one reference solver object
 *   Foam::geometricVofExt::SimPLIC::solveVofEqu
 *     (src/SimPLIC/solveVofEqu/solveVofEqu.H:67-216)
 * and runs its reconstruct() / advect() on one GPU.  Everything crosses the
 * boundary as plain pointers and sizes; the library owns its device memory,
 * never aborts and never falls back to a CPU path: every entry point returns
 * SIMPLIC_OK (0) or an error code with a message in simplic_last_error().
 *
 * Array conventions (OpenFOAM polyMesh): cells 0..n_cells-1; faces
 * 0..n_faces-1 with internal faces first (upper-triangular owner/neighbour
 * order) and boundary faces after; vectors are interleaved xyz doubles.
 * "Boundary arrays" are indexed by (face - n_internal_faces).
 */
#ifndef SIMPLIC_H
#define SIMPLIC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SIMPLIC_OK 0
#define SIMPLIC_ERR_INVALID_ARGUMENT 1
#define SIMPLIC_ERR_CUDA 2
#define SIMPLIC_ERR_MESH_CAPS 3  /* a cell or face exceeds the static caps */
#define SIMPLIC_ERR_DEVICE 4     /* a kernel reported overflow / bad data */
#define SIMPLIC_ERR_STATE 5      /* call order (e.g. advect before reconstruct) */
#define SIMPLIC_ERR_UNSUPPORTED 6

/* orientationMethod (reconstruction.C:60-68) */
#define SIMPLIC_ORIENTATION_ALPHA_GRAD 0     /* "alphaGrad": not supported */
#define SIMPLIC_ORIENTATION_ISO_ALPHA_GRAD 1 /* "isoAlphaGrad" / "LS" */
#define SIMPLIC_ORIENTATION_ISO_RDF 2        /* "isoRDF" / "RDF" (plain FP64 precision) */

/* arithmetic of the step */
#define SIMPLIC_PRECISION_PLAIN_FP64 0 /* bit-exact FP64 restatement */
#define SIMPLIC_PRECISION_MIXED 1      /* FP32 normals + Simpson clipping */
#define SIMPLIC_PRECISION_LEARNED 2    /* mixed, with the learned-normal network (simplic_set_network) */

#define SIMPLIC_MEM_HOST 0
#define SIMPLIC_MEM_DEVICE 1

/* advect flag: alpha still holds exactly what the last reconstruct saw */
#define SIMPLIC_ALPHA_UNCHANGED 1u

typedef struct simplic_handle simplic_handle;

/* The mesh as OpenFOAM holds it (fvMesh points/faces/owner/neighbour and the
 * geometric fields C, V, Cf, Sf, magSf).  Copied to the device by create. */
typedef struct simplic_mesh_desc {
    int32_t n_points;
    int32_t n_faces;
    int32_t n_internal_faces;
    int32_t n_cells;
    const double* points;         /* [3 n_points] */
    const int32_t* face_offsets;  /* [n_faces+1] CSR into face_points */
    const int32_t* face_points;   /* stored order, right-hand normal out of owner */
    const int32_t* owner;         /* [n_faces] */
    const int32_t* neighbour;     /* [n_internal_faces] */
    const double* cell_centres;   /* [3 n_cells]  mesh.C() */
    const double* cell_volumes;   /* [n_cells]    mesh.V() */
    const double* face_centres;   /* [3 n_faces]  mesh.Cf() */
    const double* face_areas;     /* [3 n_faces]  mesh.Sf() */
    const double* face_mag_areas; /* [n_faces]    mesh.magSf() */
} simplic_mesh_desc;

/* fvSolution solvers."alpha.*" keys read by the reference
 * (reconstruction.C:502-516, advection.C:455-457), same defaults. */
typedef struct simplic_controls {
    double mixed_cell_tol;       /* mixedCellTol      1e-8 */
    int32_t orientation_method;  /* orientationMethod isoAlphaGrad */
    int32_t split_warped_face;   /* splitWarpedFace   false (true: plain FP64 precision) */
    int32_t n_alpha_bounds;      /* nAlphaBounds      10 */
    double snap_tol;             /* snapTol           0 */
    int32_t clip;                /* clip              true */
    int32_t write_plic_fields;   /* writePlicFields   false (accepted, no effect) */
    int32_t map_alpha_field;     /* mapAlphaField     false (the caller maps with simplic_map_alpha_field) */
    int32_t precision;           /* SIMPLIC_PRECISION_* */
    int32_t record_cut_faces;    /* keep a per-face mask of Simpson faces */
    double iso_rdf_tol;          /* tol               1e-6 (isoRDF) */
    double iso_rdf_rel_tol;      /* relTol            0.1  (isoRDF) */
    int32_t iso_rdf_iterations;  /* iterations        5    (isoRDF) */
} simplic_controls;

/* Per-step inputs of advect.  Pointers are host or device memory as the
 * entry point states.  NULL U_boundary / alpha_boundary mean zero-gradient
 * (owner-cell value); NULL Sp / Su mean zeroField. */
typedef struct simplic_step_inputs {
    const double* phi;            /* [n_faces] face volume flux */
    const double* U;              /* [3 n_cells] cell velocity */
    const double* U_boundary;     /* [3 n_boundary_faces] or NULL */
    const double* alpha_boundary; /* [n_boundary_faces] or NULL */
    const double* Sp;             /* [n_cells] or NULL */
    const double* Su;             /* [n_cells] or NULL */
    double dt;                    /* mesh.time().deltaTValue() */
    uint32_t flags;               /* SIMPLIC_ALPHA_UNCHANGED */
} simplic_step_inputs;

/* Defaults of the reference dictionary lookups. */
void simplic_default_controls(simplic_controls* c);

/* Replaces the solveVofEqu constructor (solveVofEqu.C:55-91): uploads the
 * mesh once into structure-of-arrays CSR and computes the face flatness
 * (reconstruction.C:408-440).  stream: a cudaStream_t or NULL (a private
 * stream is created).  On failure *out is NULL and simplic_last_error(NULL)
 * holds the message. */
int simplic_create(const simplic_mesh_desc* mesh, const simplic_controls* controls, void* stream,
                   simplic_handle** out);
int simplic_destroy(simplic_handle* h);
const char* simplic_last_error(const simplic_handle* h);

/* --- drop-in entry points: host arrays, return when results are ready --- */

/* solveVofEqu::reconstruct() (solveVofEqu.C:96-99 -> reconstruction.C:680-722)
 * on alpha [n_cells].  With the isoRDF orientation the call synchronises
 * with the device once per iteration of the orientation loop (its stopping
 * test is a sum over the mixed cells in cell order), in the resident form
 * too. */
int simplic_reconstruct(simplic_handle* h, const double* alpha);

/* solveVofEqu::advect(Sp, Su) (solveVofEquTemplates.C:35-43 ->
 * advectionTemplates.C:352-418).  alpha [n_cells] is the current field on
 * entry and the advected field on return (alpha1 is modified in place);
 * alpha_old = alpha1.oldTime() or NULL when it equals the entry alpha.
 * U and U_boundary in pinned (page-locked) host memory are read in place by
 * the kernels that need them (around the interface) instead of being
 * copied. */
int simplic_advect(simplic_handle* h, double* alpha, const double* alpha_old, const simplic_step_inputs* in);

/* --- device-resident entry points (alpha stays in HBM between steps) ---
 * The calls only enqueue work on the handle's stream, and the device inputs
 * are read there: write phi, U, ... on that same stream (pass it to
 * simplic_create) or synchronise before the call.  A private stream made by
 * simplic_create is non-blocking, so work on other streams is not ordered
 * with it. */
int simplic_set_alpha(simplic_handle* h, const double* alpha, int32_t mem);
int simplic_reconstruct_resident(simplic_handle* h);
/* in: device pointers; alpha_old is the resident alpha. */
int simplic_advect_resident(simplic_handle* h, const simplic_step_inputs* in);
/* device pointer of the resident alpha (valid until the next advect) */
const double* simplic_alpha_device(const simplic_handle* h);
int simplic_get_alpha(simplic_handle* h, double* out, int32_t mem);
/* wait for the handle's stream and report device-side errors */
int simplic_synchronize(simplic_handle* h);

/* --- accessors (solveVofEqu.H:145-211, reconstruction.H:311-399) --- */

/* mixedCells() ascending with cellStatus() (-1 / 0 / +1); either output may
 * be NULL to query *n only. */
int simplic_get_mixed_cells(simplic_handle* h, int32_t* n, int32_t* cells, int32_t* status);
/* interfaceN / D / C / S as full cell fields (zero outside mixed cells) */
int simplic_get_interface(simplic_handle* h, double* n, double* d, double* c, double* s);
/* alphaPhi() = dVf / dt (advectionTemplates.C:417), [n_faces] */
int simplic_get_alpha_phi(simplic_handle* h, double* out, int32_t mem);
/* getRhoPhi(rho1, rho2) = (rho1 - rho2) alphaPhi + rho2 phi (advection.H:329-343);
 * phi and out in `mem` memory. */
int simplic_get_rho_phi(simplic_handle* h, double rho1, double rho2, const double* phi, double* out,
                        int32_t mem);
int simplic_get_face_flatness(simplic_handle* h, double* out);
/* 1 where dVf came from the Simpson integration (needs record_cut_faces) */
int simplic_get_cut_faces(simplic_handle* h, uint8_t* mask);
/* reconstructionTime / advectionTime / alphaMappingTime in seconds
 * (device time of the kernels) */
int simplic_timers(simplic_handle* h, double* reconstruction_s, double* advection_s, double* mapping_s);
/* mixed cells of the last reconstruct, bounding passes and most bounded
 * cells of the last advect */
int simplic_stats(simplic_handle* h, int32_t* n_mixed, int32_t* bound_passes, int32_t* max_bound_cells);

/* --- kernel-level timing (diagnostics; off by default) --- */

#define SIMPLIC_N_KERNELS 14
/* enable: record a CUDA event pair around every kernel launch on the
 * handle's stream (adds no synchronisation) */
int simplic_set_kernel_timing(simplic_handle* h, int32_t enable);
/* per kernel (SIMPLIC_N_KERNELS entries): summed device time in ms of the
 * timed launches, number of kernel launches made since create or the last
 * reset, and a static name; any output may be NULL.  Synchronises the
 * stream. */
int simplic_kernel_times(simplic_handle* h, double* total_ms, int64_t* launches, const char** names);
int simplic_reset_kernel_times(simplic_handle* h);
/* bounding diagnostics of the last advect: info[4] = passes run, most
 * overshooting cells in a pass, most dependency chains started from the
 * ready queue in a pass, and which bounding list overflowed (0 none,
 * 1 overshoot list, 3 modified-face list, 4 touched-cell list, 5 candidate
 * list; 2 is not produced) */
int simplic_bound_info(simplic_handle* h, int32_t* info);
/* how the bounding of the last advect ran: info[4] = most overshooting
 * cells one warp ran in a row along a dependency chain, cells run in all
 * passes, microseconds in the dependency phases and microseconds of the
 * whole bounding launch (both on the clock of its first block) */
int simplic_bound_profile(simplic_handle* h, int32_t* info);
/* reconstruction::mapAlphaField (reconstruction.C:725-784) after a mesh
 * refinement, on a handle created for the new mesh: every cell with
 * lower <= alpha <= upper (dynamicMeshDict lowerRefineLevel /
 * upperRefineLevel) gets the volume fraction that its interface plane cuts
 * from it.  normal [3 n_cells] and distance [n_cells] are the interfaceN /
 * interfaceD fields mapped onto the new mesh (a child cell carries its
 * parent's plane); alpha [n_cells] is updated in place.  All three in
 * `mem` memory.  The device time adds to the alphaMappingTime of
 * simplic_timers. */
int simplic_map_alpha_field(simplic_handle* h, double* alpha, const double* normal, const double* distance,
                            double lower, double upper, int32_t mem);

/* The PLIC surface of the last reconstruct (reconstruction::interface,
 * reconstruction.C:787-835, with cutCell::interfacePoints, cutCell.C:545-608):
 * one polygon per mixed cell whose plane cuts it, ascending in cell; polygon
 * k has the points offsets[k] .. offsets[k+1]-1 of points (xyz), ordered
 * around the interface centre, and belongs to cells[k].  Pass NULL outputs
 * to get *n_polys and *n_points; offsets holds n_polys + 1 entries.  The
 * first request after a reconstruct builds the surface on the device. */
int simplic_get_interface_polygons(simplic_handle* h, int32_t* n_polys, int32_t* n_points, int32_t* offsets,
                                   double* points, int32_t* cells);
/* iterations of the isoRDF orientation loop in the last reconstruct (0 for
 * the least-squares orientation) */
int simplic_rdf_iterations(simplic_handle* h, int32_t* n);
/* mesh structure found at create: info[5] = the common face count of all
 * cells (0 if they differ), the lattice dimensions nx, ny, nz (0 if the
 * mesh is not a single-block lattice with owner-ordered faces), and the
 * number of axis-aligned box cells */
int simplic_mesh_info(simplic_handle* h, int32_t* info);

/* --- mixed-cell scan without device allocation --- */

/* This entry point has no counterpart in the reference.  It is for callers
 * that may not call cudaMalloc where they need the interface cells: solvers
 * whose device memory belongs to their own pool or framework allocator, or
 * that run under a fixed memory budget, and so cannot create a handle.
 *
 * Writes the cells with mixed_cell_tol < alpha < 1 - mixed_cell_tol in
 * ascending order (the list simplic_get_mixed_cells gives after
 * simplic_reconstruct on the same alpha) to cells[0 .. min(n, capacity))
 * and n to *n_mixed.  alpha, cells and n_mixed are device pointers;
 * stream is a cudaStream_t or NULL; the call only enqueues work.  It
 * allocates no memory: its scratch is a fixed 256 KiB device array in the
 * library, which every device that loads the library keeps until exit, so
 * n_cells above SIMPLIC_NOALLOC_MAX_CELLS is rejected with
 * SIMPLIC_ERR_INVALID_ARGUMENT and a message in simplic_last_error(NULL).
 * The first call on a device looks up the scratch array's device address;
 * make that first call before any stream capture.  A failed lookup is not
 * remembered (the next call tries again); the address found is kept for
 * the life of the process, so the entry point must not be used on a
 * device after cudaDeviceReset.  All calls on a device
 * share the scratch, so calls that overlap on the GPU (other streams, other
 * host threads) race: order them on one stream or synchronise between them. */
#define SIMPLIC_NOALLOC_MAX_CELLS 134217728
int simplic_mixed_cells_noalloc(const double* alpha, int32_t n_cells, double mixed_cell_tol, int32_t* cells,
                                int32_t capacity, int32_t* n_mixed, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SIMPLIC_H */
