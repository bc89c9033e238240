// C API of the host hierarchy producer (hho_gen.cpp): the condensed HHO face system and the
// geometric multigrid hierarchy of fhhos4's in-house square/cube meshes. Arrays returned by
// the accessors are owned by the handle and stay valid until fhg_hho_destroy.
#ifndef FHG_HHO_GEN_H
#define FHG_HHO_GEN_H
#ifdef __cplusplus
extern "C" {
#endif

#define FHG_HHO_SOURCE_SINE 0      /* f = d pi^2 prod sin(pi x_i), u = prod sin(pi x_i) */
#define FHG_HHO_SOURCE_ONE 1       /* f = 1 */
#define FHG_HHO_SOURCE_RANDOM_MODES 2 /* f = sum of 4 modes a_i prod_d sin(pi m_id x_d), m_id uniform in
                                        {1..4}, a_i ~ N(0, 1), from the seed */
#define FHG_HHO_IDENTITY 0         /* K = I */
#define FHG_HHO_CHECKERBOARD 1     /* isotropic, m^d checkerboard alternating 1 and `contrast` */
#define FHG_HHO_ANISOTROPIC 2      /* per m^d block: R diag(1,..,1,eps) R^T, eps log-uniform in
                                      [eps_min, 1], R a random rotation (seeded splitmix64) */
#define FHG_HHO_LOGNORMAL_PATCHES 3 /* isotropic, per m^d block kappa log-uniform in
                                      [1/contrast, contrast] (seeded) */

typedef struct {
    int dim;              /* 2: unit square, 2 triangles per cell; 3: unit cube, 6 tetrahedra per cube */
    int n;                /* cells per direction */
    int k;                /* face polynomial degree (1..3) */
    int max_coarse_rows;  /* coarsen while the level has more rows (MatrixMaxSizeForCoarsestLevel) */
    int max_levels;       /* > 0: fixed number of levels instead */
    int source;           /* FHG_HHO_SOURCE_* */
    int coefficient;      /* FHG_HHO_IDENTITY / FHG_HHO_CHECKERBOARD */
    double contrast;
    int checker_blocks;   /* m (4) */
    int threads;          /* 0: all hardware threads */
    double eps_min;       /* FHG_HHO_ANISOTROPIC: smallest eps (1e-3) */
    unsigned long long seed; /* coefficient fields and random sources */
    int p_tables;         /* 1: keep the tables of every P (fhg_hho_prolongation_tables); 0 (default) */
} fhg_hho_params;

typedef struct fhg_hho fhg_hho;

void fhg_hho_default_params(fhg_hho_params* p);
int fhg_hho_create(fhg_hho** h, const fhg_hho_params* p);
void fhg_hho_destroy(fhg_hho* h);
const char* fhg_hho_last_error(const fhg_hho* h);
int fhg_hho_num_levels(const fhg_hho* h);
int fhg_hho_block_size(const fhg_hho* h);
int fhg_hho_level(const fhg_hho* h, int level, int* n_rows, long long* nnz, const int** rowptr,
                  const int** colidx, const double** vals);
int fhg_hho_prolongation(const fhg_hho* h, int level, int* n_rows, int* n_cols, long long* nnz,
                         const int** rowptr, const int** colidx, const double** vals);
int fhg_hho_rhs(const fhg_hho* h, const double** b);
/* The tables of P_l (kept with p_tables = 1; -2 otherwise), for assembling it elsewhere: a coarse
 * element's contribution to a fine face depends only on the element's class and the face's place
 * in it, so it is stored once per such slot. Sizes, then the arrays (each optional): face_ce and
 * face_w [n_face_blocks * 2] (the unknown fine face's coarse elements, -1 for none, and their
 * weights), face_slot [n_face_blocks * 2], slot_contrib [n_slots * bs * faces_per_element * bs]
 * (row-major bs x faces_per_element*bs per slot), coarse_elem_faces [n_coarse_elements *
 * faces_per_element] (coarse unknown blocks, -1: Dirichlet). P's block row of face I sums, over its
 * coarse elements t, face_w * slot_contrib with column block lf of the slot going to coarse block
 * coarse_elem_faces[ce][lf]. */
int fhg_hho_prolongation_table_sizes(const fhg_hho* h, int level, int* n_face_blocks, int* n_slots,
                                     int* n_coarse_elements, int* block_size, int* faces_per_element);
int fhg_hho_prolongation_tables(const fhg_hho* h, int level, int* face_ce, double* face_w, int* face_slot,
                                double* slot_contrib, int* coarse_elem_faces);
/* Relative L2 error of the reconstruction of face solution x (level-0 numbering) against the
 * exact solution of the sine source; -2 for sources without a closed form. */
int fhg_hho_l2_error(const fhg_hho* h, const double* x, double* rel_error);
/* Post-processing tables of the finest level: sizes (n_face_dofs = faces per element x face DOFs,
 * n_points = cell quadrature points of the L2 error), then the arrays, each optional (null: skipped):
 * elem_class[ne], elem_faces[ne * (dim + 1)] (unknown block or -1), elem_centre[ne * 3],
 * cell_rhs[ne * n_cell] (A_TT^-1 b_T), and per class solve_cells[n_cell * n_face_dofs] (-A_TT^-1 A_TF),
 * recon[n_recon * (n_cell + n_face_dofs)], weights[n_points], offsets[n_points * 3] (from the centroid),
 * basis[n_points * n_recon]. */
int fhg_hho_post_sizes(const fhg_hho* h, int* n_elements, int* n_classes, int* n_cell, int* n_face_dofs,
                       int* n_recon, int* n_points);
int fhg_hho_post_tables(const fhg_hho* h, int* elem_class, int* elem_faces, double* elem_centre, double* cell_rhs,
                        double* solve_cells, double* recon, double* weights, double* offsets, double* basis);
/* Inputs of static condensation on the finest level: local[n_classes * nH * nH] (nH = n_cell +
 * n_face_dofs; the local operator before condensation, cells first), b_cell[ne * n_cell] (b_T),
 * face_elems[n_face_blocks * 4] = (e1, lf1, e2, lf2) per unknown face block, in assembly order. */
int fhg_hho_condense_tables(const fhg_hho* h, double* local, double* b_cell, int* face_elems);
/* The same condensation inputs for any level (each level is rediscretised on its own mesh; no source
 * term): sizes, then elem_class[ne], elem_faces[ne * (dim + 1)], local[n_classes * nH * nH],
 * face_elems[n_face_blocks * 4]; null arrays are skipped. */
int fhg_hho_level_sizes(const fhg_hho* h, int level, int* n_elements, int* n_classes, int* n_cell,
                        int* n_face_dofs, int* n_face_blocks);
int fhg_hho_level_tables(const fhg_hho* h, int level, int* elem_class, int* elem_faces, double* local,
                         int* face_elems);
/* Diffusion tensors of the two elements of every unknown face of level `level` (both exist: the
 * unknowns are the interior faces): out[12*u .. 12*u+11] for face block u, element 1 then
 * element 2 (the face's own element order), each as (xx, yy, zz, xy, xz, yz) in 3D and
 * (xx, yy, xy, 0, 0, 0) in 2D. */
int fhg_hho_face_tensors(const fhg_hho* h, int level, double* out);

#ifdef __cplusplus
}
#endif
#endif
