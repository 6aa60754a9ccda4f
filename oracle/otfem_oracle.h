/*
 * otfem_oracle.h -- CPU oracle for the stiffness-warped tetrahedral FEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of OpenTissue's
 * fem::init / fem::simulate (OpenTissue/dynamics/fem/*.h) used as the checker
 * for the CUDA library and as the timed CPU baseline.  Nothing in the product
 * path links or calls it.  Every function keeps the reference's floating-point
 * operation order (compile with -ffp-contract=off) so that its results are
 * bit-identical to the reference headers compiled with the same flags.
 *
 * The same C interface is exported by the reference-backed build under
 * oracle/_ref (oracle/ref/ref_capi.cpp), so tests can run both side by side.
 */
#ifndef OTFEM_ORACLE_H
#define OTFEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh orc_mesh;

/* Node fields for orc_set_field / orc_get_field (3 doubles per node unless noted). */
enum {
  ORC_COORD = 0,       /* m_coord */
  ORC_MODEL_COORD = 1, /* m_model_coord */
  ORC_VELOCITY = 2,    /* m_velocity */
  ORC_F_EXTERNAL = 3,  /* m_f_external */
  ORC_MASS = 4,        /* m_mass (1 double per node, get only) */
  ORC_F0 = 5,          /* m_f0 (get only) */
  ORC_B = 6            /* m_b (get only) */
};

/* Mesh generator: t4mesh_block_generator.h:32-110.  tets: 4*5*I*J*K ints,
 * coord: 3*(I+1)*(J+1)*(K+1) doubles. */
void orc_generate_blocks(int I, int J, int K, double w, double h, double d, int *tets, double *coord);

orc_mesh *orc_create(int n_nodes, int n_tets, const int *tets, const double *coord,
                     const double *model_coord, const unsigned char *fixed);
void orc_destroy(orc_mesh *m);
void orc_set_fixed(orc_mesh *m, const unsigned char *fixed);
void orc_set_field(orc_mesh *m, int field, const double *src);
void orc_get_field(orc_mesh *m, int field, double *dst);

/* fem::init (fem_init.h:45-65). */
void orc_init(orc_mesh *m, double young, double poisson, double density, double c_yield,
              double c_creep, double c_max);
/* fem::simulate (fem_simulate.h:49-113): 20-iteration CG, mass damping 2.0. */
void orc_simulate(orc_mesh *m, double dt, int use_warping);
/* Same pipeline with the CG replaced by a clamp-free relative-residual CG that
 * stops when ||r|| <= rtol*||b|| over free rows (big_conjugate_gradient.h:92-94
 * rule, measured against b).  Returns iterations and the final true relative
 * residual ||b - A v|| / ||b||. */
void orc_simulate_converged(orc_mesh *m, double dt, int use_warping, double mass_damping,
                            double rtol, int max_iterations, int *iterations, double *rel_residual);
/* fem::update_original_coord (fem_update_original_coord.h:28-33). */
void orc_update_original_coord(orc_mesh *m);

/* fem::export_K (fem_export_k.h:23-68) as (row, col, value) triplets in push order. */
long orc_export_k_count(orc_mesh *m);
void orc_export_k(orc_mesh *m, int *rows, int *cols, double *vals);

/* The node K_row maps: key sets (CSR, ascending columns) and 3x3 values. */
long orc_k_nnz(orc_mesh *m);
void orc_k_pattern(orc_mesh *m, int *row_ptr, int *cols);
void orc_k_values(orc_mesh *m, double *vals);

/* Per-tet state: m_Re (9, row-major), m_plastic (6), m_V (1). */
void orc_get_re(orc_mesh *m, double *re);
void orc_get_plastic(orc_mesh *m, double *plastic);
void orc_get_volume(orc_mesh *m, double *vol);

#ifdef __cplusplus
}
#endif
#endif
