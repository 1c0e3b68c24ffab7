/*
 * nmag_gpu.h -- C-ABI of libnmaggpu.so: a GB300 (sm_103a) implementation of
 * nsim's LLG right-hand side and its time integration.
 *
 * The reference exposes this path to Python through the embedded "ocaml"
 * module (src/nsimexec.ml:4467-4674).  Each entry point below names the
 * reference call it replaces.  Conventions: every function returns an int
 * status (0 = ok, < 0 = invalid argument, > 0 = numerical failure such as a
 * solver iteration cap or non-finite values); nothing aborts or traps.  The
 * handle owns all device memory; the caller owns host arrays, which are
 * copied in and out.  Handles are not thread-safe; use one per thread.
 *
 * Units: simulation units throughout (m = 1e-9, s = 1e-12, A = 1e-3,
 * kg = 1e-27; interface/nmag/main.py:188-196).  Vector fields are node-major,
 * component-minor (dof = 3*node + c), which is the reference's DOF order for
 * one material covering the mesh (src/fem.ml:2592-2720).
 */
#ifndef NMAG_GPU_H
#define NMAG_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NMG_VERSION 10000

typedef struct nmg_handle nmg_handle;

/* Material constants in simulation units, as the reference's local equations
 * and operator strings see them (interface/nmag/main.py:347-465,
 * interface/nmag/nmag_lam.py:417-460). */
typedef struct nmg_material {
  double Ms;            /* su_Ms                                                  */
  double exch_coeff;    /* su_exch_prefactor = 2A/(mu0 Ms)                        */
  double C1, C2, C3;    /* LLG coefficients: C1 m x H + C2 m x (m x H) + C3 (1-m.m) m */
  double K1;            /* uniaxial anisotropy constant (su); 0 = none            */
  double axis[3];       /* unit easy axis                                         */
  double anis_coeff;    /* 2 K1 / (mu0 Ms)                                        */
  double E_coeff_half;  /* -0.5 Ms mu0 (exchange and demag energy densities)      */
  double E_coeff_ext;   /* -1.0 Ms mu0 (Zeeman energy density)                    */
} nmg_material;

/* Solver and precision options (nmag.Simulation(...) kwargs, main.py:829-845,
 * and the ksp_tolerances of nmag_lam.py:614-634). */
typedef struct nmg_options {
  int do_demag;                          /* 0: skip FEM/BEM demag                      */
  double nbc_rtol, nbc_atol; int nbc_maxits;   /* Neumann Poisson solve              */
  double dbc_rtol, dbc_atol; int dbc_maxits;   /* Dirichlet Poisson solve            */
  int bem_precision;                     /* 0: FP64 matrix; 1: FP32 matrix, FP64 sums;
                                            2: FP32 + BF16-residual matrix, compensated
                                               FP32 products (~2^-44);
                                            3: tensor cores: B and x split into three
                                               BF16 planes each, six tcgen05 products
                                               per term, FP32 sums over 2048 terms
                                               added in FP64 (~2^-24); an ensemble's
                                               members form one product              */
  int cg_precision;                      /* 0: FP64 CG; 1: FP32 inner CG (two-level for
                                            the Neumann system, warm-started from the
                                            last solves) with FP64 residual refinement
                                            to the same tolerance                     */
  int cg_no_coarse;                      /* 1: Jacobi only (no two-level Neumann CG)   */
  int n_members;                         /* ensemble size B (0 or 1: one simulation)   */
  double bem_anchor_tol;                 /* bem_precision 2 only; > 0: anchored product
                                            y = B x0 + B32 (x - x0) while
                                            max|x - x0| <= tol max|x| per member, a new
                                            compensated anchor otherwise; 0: off
                                            (finite, >= 0)                             */
  int adjoint_cg_precision;              /* Poisson solves of nmg_rk4_adjoint's backward
                                            pass: 0 FP64 CG; 1 FP32 CG with FP64 residual
                                            refinement (to the same tolerance)         */
  int anchor_product;                    /* anchored ensemble product's difference
                                            B (x - x0): 0 FP32 copy of B; 1 FP16 copy of
                                            B in tensor-core fragment order (FP32
                                            accumulation; ~2^-11 of |B||x - x0|)        */
  int cg_local_sweeps;                   /* FP32 inner CG (cg_precision 1): damped Jacobi
                                            sweeps on each thread block's own rows in
                                            the preconditioner (0 or 1: Jacobi alone) */
  int jv_precision;                      /* the BDF's Jacobian-vector products and block
                                            preconditioner at Jacobian level 0: 0 FP64;
                                            1 FP32 arithmetic on FP32 copies of the
                                            frozen state, the exchange matrix and the
                                            direction (the Newton matrix only: the
                                            residual stays FP64)                      */
} nmg_options;

/* Integrator statistics (CVODE counters; nsim.ml:354-387 timings). */
typedef struct nmg_ts_stats {
  int64_t nst, nfe, nni, nli, ncfn, netf, npe, nps, njv, nje;
  double hcur, tcur;
  int32_t qcur, last_cg_iters_nbc, last_cg_iters_dbc, pad;
  double time_rhs_ms, time_jv_ms, time_psolve_ms;
} nmg_ts_stats;

/* Library version; replaces nothing (ocaml.version). */
int nmg_version(void);

/* Select the GPU for the handles this thread creates next (the library keeps
 * its own CUDA runtime state: the caller's own cudaSetDevice or a framework's
 * device choice does not carry over).  No counterpart in the reference. */
int nmg_set_device(int device);

/* Message of the last failing call on this handle (or, when h == NULL, of the
 * last failing nmg_create or handle-less call on this thread). */
const char *nmg_last_error(const nmg_handle *h);

/* Build the mesh topology, the P1 CSR operators, the box volumes, the surface
 * triangles, solid angles and the dense Lindholm BEM on the device.
 * Replaces ocaml.raw_make_lam -> Nsim.make_linalg_machine (nsimexec.ml:3605,
 * nsim.ml:2828-3150): operator vivification (fem.ml:4890-5366) and the BEM
 * fill (bem3d.ml:938-1047, bem3d_stubs.c:413-610). */
int nmg_create(const double *coords, int n_nodes, const int32_t *tets, int n_tets,
               const nmg_material *mat, const nmg_options *opt, nmg_handle **out);

/* Release every device resource of the handle. */
int nmg_destroy(nmg_handle *h);

/* Sizes: info[0..5] = N, T, nnz (scalar P1 pattern), Nb, number of surface
 * triangles, number of outer faces. */
int nmg_mesh_info(const nmg_handle *h, int64_t info[6]);

/* Copy the scalar P1 CSR and its value arrays (K, G_x|G_y|G_z, D_x|D_y|D_z,
 * box volumes) to the host.  Any pointer may be NULL. */
int nmg_get_csr(const nmg_handle *h, int32_t *row_ptr, int32_t *col_idx, double *K, double *G3,
                double *D3, double *vol);

/* Reference-shaped CSR of one of the six operators of nmag_lam.py:569-606:
 * which = 0 op_H_exch (3N x 3N), 1 op_div_m (N x 3N), 2 op_neg_laplace_phi
 * (N x N), 3 op_grad_phi (3N x N), 4 op_laplace_DBC (N x N), 5 op_load_DBC
 * (N x Nb); entries scaled by coeff.  Built on the device from the scalar
 * pattern.  Call with NULL arrays to query rows/cols/nnz first. */
int nmg_export_operator(const nmg_handle *h, int which, double coeff, int *rows, int *cols, int *nnz,
                        int32_t *row_ptr, int32_t *col_idx, double *vals);

/* Boundary data: node of each boundary short index (Nb), surface triangles
 * (3 per triangle, short indices), outward unit normals (3 per triangle),
 * interior solid angles (Nb).  Any pointer may be NULL. */
int nmg_get_boundary(const nmg_handle *h, int32_t *node_of_b, int32_t *tri, double *tri_normal,
                     double *solid_angle);

/* Dense BEM matrix, row-major Nb x Nb (row = observer). */
int nmg_get_bem(const nmg_handle *h, double *out);

/* Magnetisation (3N); replaces ocaml.lam_set_field/lam_get_field on v_m
 * (nsimexec.ml:4286).  set_m copies as given (normalise on the host, as
 * Fields.set_subfield does with auto_normalise, main.py:635-705). */
int nmg_set_m(nmg_handle *h, const double *m);
int nmg_get_m(const nmg_handle *h, double *m);

/* Applied field H_ext (3N, su); v_H_ext of nmag_lam.py:358. */
int nmg_set_h_ext(nmg_handle *h, const double *h_ext);

/* Replace the material constants (e.g. the damping between a relax stage
 * and the dynamics); invalidates the integrator like the reference's
 * reinitialise. */
int nmg_set_material(nmg_handle *h, const nmg_material *mat);

/* A general anisotropy in the polynomial form the reference generates for it
 * (src/nsim_anisotropy.ml:207-236 anisotropy_equations, called from
 * interface/nmag/nmag_lam.py:485-502 for every anisotropy other than the
 * closed-form uniaxial K1 term of nmg_material):
 *   E_anis   = sum_{t < n_e} e_coef[t] mx^a my^b mz^c,       a,b,c from e_pow[t]
 *   H_anis,d = sum_{t < n_h} h_coef[3t + d] mx^a my^b mz^c,  a,b,c from h_pow[t]
 * with the exponents packed a | b << 4 | c << 8 (each 0..13) and at most 1024
 * terms each.  The host forms both polynomials (fit of the energy on the unit
 * sphere, tangential gradient times -1/(mu0 Ms)); the field is added to the
 * K1 term (set K1 = 0 to use the polynomial alone) in every member of an
 * ensemble.  n_e = n_h = 0 removes it.  Invalidates the integrator.  The RK4
 * adjoint refuses handles with a polynomial anisotropy (-2). */
int nmg_set_anisotropy_poly(nmg_handle *h, int n_e, const int32_t *e_pow, const double *e_coef, int n_h,
                            const int32_t *h_pow, const double *h_coef);

/* Spin-transfer torque (Zhang-Li form of interface/nmag/nmag_lam.py:417-424,
 * 872-903): dm/dt gains c4 m x (m x u) + c5 m x u with u = dm_dcurrent =
 * (J . grad) m, computed every RHS as G_j m (the op_grad_phi pattern without
 * its sign) dotted with the current density J per node and divided by the box
 * volume.  c4 = su_llg_stt_adiab, c5 = su_llg_stt_nadiab of the material
 * (main.py:440-451), rounded like the other LLG coefficients; 0, 0 switches
 * it off.  The timestepper's Jacobian ignores these terms, as the
 * reference's (nmag_lam.py:432-436).  The RK4 adjoint refuses a handle with
 * it switched on (-2). */
int nmg_set_stt(nmg_handle *h, double c4, double c5);

/* Current density J (3N per member, simulation units of A/m^2; NULL = zero),
 * v_current_density of main.py:1934-1960.  Invalidates the integrator. */
int nmg_set_current_density(nmg_handle *h, const double *j);

/* Pinning field (N values, one per node, shared by the members of an
 * ensemble; NULL = 1 everywhere): the factor `pin` of every term of dm/dt and
 * of the timestepper's Jacobian rows (interface/nmag/nmag_lam.py:417-436;
 * Simulation.set_pinning, main.py:1918-1935).  0 fixes the magnetisation of a
 * node.  Invalidates the integrator.  The RK4 adjoint refuses a handle with a
 * pinning field (-2). */
int nmg_set_pinning(nmg_handle *h, const double *pin);

/* Evaluate the RHS at the current m (program update_dmdt, nmag_lam.py:784-
 * 795) and copy fields out: fields = [H_exch | H_demag | H_anis | H_total |
 * dmdt] (5 x 3N), scalars = [phi | rho] (2 x N).  Either may be NULL. */
int nmg_eval_fields(nmg_handle *h, double *fields, double *scalars);

/* Energy densities [E_exch | E_demag | E_ext | E_anis | E_total] (5 x N) at
 * the current m (program update_E, nmag_lam.py:454-460,659-662). */
int nmg_energy_density(nmg_handle *h, double *E5);

/* Volume averages of m (3) and total energies (5) = sum_i E_i V_i
 * (main.py:2313-2480, fem.ml:3246-3283). */
int nmg_averages(nmg_handle *h, double avg_m[3], double energies[5]);

/* Ensemble (options n_members = B > 1): B independent simulations on the same
 * mesh and material, integrated as one ODE system.  Every per-node array of
 * the calls above then holds B member blocks, member b at offset b * 3N (or
 * b * N for scalars; energy densities [k][member][node]); nmg_averages
 * reports member 0 and this call any member.  No counterpart in the
 * reference, which runs one simulation per process. */
int nmg_member_averages(nmg_handle *h, int member, double avg_m[3], double energies[5]);

/* Several magnetic materials (main.py:1182-1191 region -> material mapping;
 * nmag_lam.py:183-470 one m field per material).  Replaces ocaml.raw_make_lam
 * for a mesh whose regions carry different materials.  tet_region[t] in
 * 1..n_regions is the region of tetrahedron t (vacuum simplices are not
 * passed); region r carries the materials region_mats[region_ptr[r-1] ..
 * region_ptr[r]) (indices into mats).  Every material X has its own m_X on
 * its sites -- the nodes of the simplices of its regions -- so a node on an
 * interface carries one m per material, and the exchange acts within each
 * material only; the demagnetising potential lives on every node and sees
 * all materials' charges.  Sites are numbered material by material (mats
 * order), nodes ascending within a material: nmg_mesh_info reports the site
 * count as info[0], and every per-node array of the calls above (m, H_ext,
 * fields, energies, pinning) then holds one entry per site.  Options as
 * nmg_create (precision forms, ensembles); closed-form uniaxial anisotropy
 * per material; polynomial anisotropy, spin-transfer torque and element
 * parameters are refused. */
int nmg_create_materials(const double *coords, int n_nodes, const int32_t *tets, int n_tets,
                         const int32_t *tet_region, int n_regions, const int32_t *region_ptr,
                         const int32_t *region_mats, const nmg_material *mats, int n_mats,
                         const nmg_options *opt, nmg_handle **out);
/* Local magnetic coupling between two materials whose sites share nodes
 * (two magnetic species in one crystal, e.g. the sublattices of DyFe2):
 * replaces Simulation.set_local_magnetic_coupling (main.py:1234-1263) and
 * its generated local equations (nmag_lam.py:16-62).  At every node that
 * carries both, H_lc of mat1 gains h_coeff m_mat2 (added to H_total) and
 * E_lc of mat1 gains e_coeff m_mat1 . m_mat2 (added to E_total); call it
 * once per ordered pair.  The timestepper's Jacobian leaves it out, as the
 * reference's does. */
int nmg_set_local_coupling(nmg_handle *h, int mat1, int mat2, double h_coeff, double e_coeff);
/* The mesh node and the material of every site (n_sites entries each). */
int nmg_site_info(const nmg_handle *h, int32_t *site_node, int32_t *site_material);
/* Change material k's constants (e.g. its damping between relax and dynamics). */
int nmg_set_site_material(nmg_handle *h, int material, const nmg_material *mat);
/* <m> of one material (volume average over its sites) and its energies
 * (sum of E_i V_i over its sites: exchange, demag, Zeeman, anisotropy,
 * total), of ensemble member `member`; one material: material 0 is the
 * mesh (main.py:2313-2480 averages per material). */
int nmg_material_averages(nmg_handle *h, int material, int member, double avg_m[3], double energies[5]);

/* Timestepper (re)initialisation at t0 from the current m; replaces
 * ocaml.lam_ts_init -> timestepper_set_initial_from_phys (nsim.ml:2485-2535). */
int nmg_ts_init(nmg_handle *h, double t0, double rtol, double atol, int max_order, int krylov_max);

/* Advance to t_final (CV_NORMAL_TSTOP when exact_tstop, else CV_NORMAL with
 * interpolated output), or stop after max_steps steps when max_steps >= 0
 * (CV_ONE_STEP_TSTOP loop).  m is updated to the returned time.  Replaces
 * ocaml.lam_ts_advance -> timestepper_advance -> My_CVode_Advance_Time
 * (nsimexec.ml:4130, nsim.ml:3641, sundials_sp_stubs.c:1239-1310). */
int nmg_ts_advance(nmg_handle *h, double t_final, int exact_tstop, int64_t max_steps, double *t_reached,
                   nmg_ts_stats *stats);

/* max_i |m_i - m_prev_i| over nodes (Euclidean norm of the 3-vector); the
 * reference's mwe_norm_dist_fun (nsimexec.ml:2332-2368, fem.ml:4717-4793). */
int nmg_max_dm(nmg_handle *h, const double *m_prev, double *out);
/* The same distance between the current m and m at the previous call (or at
 * the last nmg_set_m, whichever came later), without a host copy; then
 * remembers the current m.  0 on the first call after nmg_create.  Serves
 * the convergence check after each advance (main.py:1383-1455). */
int nmg_max_dm_step(nmg_handle *h, double *out);

/* Device-pointer entry points (pointers are CUDA device addresses, e.g. from
 * torch tensors): one RHS evaluation dmdt = f(m) on the handle's stream and
 * one fixed-step RK4 trajectory.  No host copies.  */
int nmg_rhs_device(nmg_handle *h, const double *d_m, double *d_dmdt);
/* y_n = B x_n for n_rhs boundary vectors (device arrays, member-major: x_n at
 * d_x + n * nb) with the handle's BEM in its bem_precision form -- the
 * reference's dense BEM MatMult (nsim.ml:3128-3140) for many right-hand sides
 * at once (with bem_precision 3 one tensor-core product).  On the handle's
 * stream; returns after the product is complete.  Not with the anchored
 * product. */
int nmg_bem_apply(nmg_handle *h, const double *d_x, double *d_y, int n_rhs);
int nmg_rk4_device(nmg_handle *h, double *d_m, double dt, int nsteps);

/* The Jacobian of the BDF's Newton iteration.  The reference's is
 * approximate: the derivative of C1 m x H + C2 m x (m x H) with H frozen plus
 * the exchange operator's dH/dm, nothing else (nmag_lam.py:665-704; its
 * do_anisotropy_jacobian adds a plan the timestepper never uses,
 * nmag_lam.py:684-693).  level 0 is that Jacobian (the default); level 1
 * adds the local terms: the anisotropy field's derivative (uniaxial, per
 * element or polynomial), the C3 length term's, and with several materials
 * the local couplings; level 2 adds the demag field's response, the demag
 * field of each Krylov direction from one Neumann + BEM + Dirichlet pipeline
 * at Poisson tolerance demag_rtol (in (0, 1)) on buffers of its own (with
 * the plain FP32 BEM product where the handle has an FP32 plane).  The
 * block-Jacobi preconditioner takes the local terms from level 1 on.  The
 * spin-torque terms are in none.  Changes the Newton iteration only: the
 * solution is the same to the integrator's tolerances. */
int nmg_set_jacobian(nmg_handle *h, int level, double demag_rtol);
/* d_out = J(d_m) d_v at the handle's level (device arrays, 3 per node or site
 * and member): one RHS evaluation at d_m for the frozen field, then the
 * Jacobian-vector product.  For tests of the Newton matrix against finite
 * differences of nmg_rhs_device. */
int nmg_jacobian_apply(nmg_handle *h, const double *d_m, const double *d_v, double *d_out);

/* Differentiation form.  No counterpart in the reference, whose material
 * constants are one scalar Ms and K1 per material (main.py:347-465); these
 * entry points extend its RHS (nmag_lam.py:734-832) with per-element weights,
 * all DEVICE arrays of n_tets doubles (NULL = all ones, or for kappa all
 * zeros):
 *   exchange  H_exch_i = -exch_coeff/V_i sum_j (sum_T wK_T K_T)_ij m_j
 *   charge    rho_i = Ms sum_T wD_T int_T grad phi_i . m
 *   anisotropy H_anis_i = c_i (a.m)(a - (a.m) m), c_i = sum_T kappa_T |T|/4 / V_i
 * With wK = Ms/Ms_T, wD = Ms_T/Ms and kappa = 2 K1_T/(mu0 Ms_T) this is a
 * per-element Ms_T and K1_T (wK = wD = 1 gives the plain model).  The weights
 * apply to every later RHS evaluation (also nmg_ts_advance) until cleared. */
int nmg_set_element_params(nmg_handle *h, const double *d_wK, const double *d_wD, const double *d_kappa,
                           const double axis[3]);
int nmg_clear_element_params(nmg_handle *h);

/* Fixed-step RK4 trajectory from d_m0 (device, 3N) over nsteps steps of dt,
 * with a checkpoint of m every ckpt_every steps kept on the device for
 * nmg_rk4_adjoint.  The applied field of step n is the handle's H_ext plus
 * the uniform pulse d_pulses[3k..3k+2] (device) with k = n / steps_per_pulse
 * (no pulse once k >= n_pulses).  Writes m after the last step to d_m_final and,
 * when d_avg_hist is not NULL, the volume average <m> after every step
 * (nsteps x 3, device). */
int nmg_rk4_forward(nmg_handle *h, const double *d_m0, double dt, int nsteps, int ckpt_every, const double *d_pulses,
                    int n_pulses, int steps_per_pulse, double *d_m_final, double *d_avg_hist);

/* Discrete adjoint of the last nmg_rk4_forward on this handle: given the
 * cotangents of m_final (3N) and of the <m> history (nsteps x 3; either may
 * be NULL), writes the gradients with respect to m0 (3N), the element weights
 * wK, wD, kappa (n_tets each) and the pulses (3 x n_pulses).  Output pointers
 * may be NULL; all are device arrays.  Element parameters and H_ext must be
 * those of the forward call. */
int nmg_rk4_adjoint(nmg_handle *h, const double *d_m_final_bar, const double *d_avg_hist_bar, double *d_m0_bar,
                    double *d_wK_bar, double *d_wD_bar, double *d_kappa_bar, double *d_pulses_bar);

/* Batching form: many independent particles (each its own mesh, material
 * and applied-field direction) advanced together in one persistent launch.
 * No counterpart in the reference (one simulation per process); each particle
 * follows the RHS of nmag_lam.py:734-832 and the hysteresis loop of
 * hysteresis.py:244-557 (relax to max |dm/dt| < stop_dmdt twice in a row,
 * then the next field H_k = h_max (1 - 2k/(n_stages-1)) along h_dir).  Time
 * integration: embedded Bogacki-Shampine 3(2) with per-particle step control
 * (or a fixed step when fixed_dt > 0).  The BEM blocks are FP32 with FP64 row
 * sums.  Arrays of all particles are concatenated in particle order. */
typedef struct nmg_particle {
  const double *coords;   /* 3 n_nodes, simulation units */
  int n_nodes;
  const int32_t *tets;    /* 4 n_tets */
  int n_tets;
  nmg_material mat;
  double h_dir[3];        /* direction of the field sweep */
} nmg_particle;

typedef struct nmg_batch_options {
  double cg_rtol; int cg_maxits;          /* both Poisson solves                         */
  int n_stages;                           /* fields in the sweep                         */
  double rtol, atol;                      /* step control (max norm)                     */
  double stop_dmdt;                       /* convergence, su (1 deg/ns = 1.745e-5)       */
  double h_max;                           /* sweep amplitude, su                         */
  double dt0, dt_max, fixed_dt;           /* initial / maximal step; fixed_dt > 0: no control */
  int threads;                            /* CTA size (0: 256)                           */
  double budget;                          /* work per particle per launch (0: one step)  */
  int integrator;                         /* 0: Bogacki-Shampine 3(2), explicit;
                                             1: ROS2, linearly implicit (L-stable) with
                                                BiCGSTAB solves of I - gamma tau J    */
  int krylov_maxits;                      /* ROS2 linear-solve cap (0: 200)              */
  int reserved[2];
} nmg_batch_options;

typedef struct nmg_batch nmg_batch;
const char *nmg_batch_last_error(const nmg_batch *b);
int nmg_batch_create(const nmg_particle *parts, int n, const nmg_batch_options *opt, nmg_batch **out);
int nmg_batch_destroy(nmg_batch *b);
int nmg_batch_info(const nmg_batch *b, int64_t *nodes_total, int32_t *nodes, int32_t *nb);
int nmg_batch_set_m(nmg_batch *b, const double *m);
int nmg_batch_get_m(const nmg_batch *b, double *m);
/* dm/dt and H_total of every particle at its current m and stage field. */
int nmg_batch_eval(nmg_batch *b, double *dmdt, double *h_total);
/* Replay a CUDA graph of `launches` persistent launches; returns when done. */
int nmg_batch_run(nmg_batch *b, int launches);
int nmg_batch_state(const nmg_batch *b, double *t, int32_t *stage, int64_t *steps, int64_t *rhs_evals,
                    int32_t *done, double *max_dmdt);
/* CTA size and per-launch work budget; the autotuner times candidates on the
 * batch (state restored afterwards) and keeps the fastest. */
int nmg_batch_set_schedule(nmg_batch *b, int threads, double budget);
int nmg_batch_autotune(nmg_batch *b, int trial_launches, int *threads_out, double *budget_out);

/* Wall-clock split of the last nmg_ts_advance / RHS work, in ms (CUDA events). */
int nmg_get_timings(const nmg_handle *h, double out[8]);

/* Measurement hooks (no counterpart in the reference; they replace the
 * TSTART/TSTOP timers of nsim.ml:3414-3455).  While profiling is enabled,
 * CUDA events bracket every launch of the hot kernels on the handle's stream:
 * kernel 0 = BEM matrix-vector product, 1 = Neumann CG, 2 = Dirichlet CG,
 * 3 = fused H_eff + LLG node kernel, 4 = Jacobian-vector + preconditioner,
 * 5 = FP32 difference product of the anchored BEM product (bem_anchor_tol).
 * nmg_profile(h, 1) clears and starts, nmg_profile(h, 0) stops;
 * nmg_profile_read returns launches and summed device milliseconds.
 * nmg_launch_count returns the number of kernels this handle has launched. */
int nmg_profile(nmg_handle *h, int enable);
int nmg_profile_read(nmg_handle *h, int kernel, int64_t *launches, double *total_ms);
int64_t nmg_launch_count(const nmg_handle *h);
/* Total CG iterations since nmg_create: [Neumann, Dirichlet] (the reference
 * reports KSP iteration counts through PETSc logging, nsim.ml:2462-2478). */
int nmg_cg_iterations(const nmg_handle *h, int64_t total[2]);
/* Anchored BEM product counters since nmg_create: [products, anchor refreshes
 * (compensated products)]; zeros when bem_anchor_tol is off.  No counterpart
 * in the reference. */
int nmg_bem_anchor_stats(const nmg_handle *h, int64_t out[2]);

/* max over nodes of |m_i - m_prev_i| for device arrays d_m, d_m_prev (3 x
 * n_nodes doubles each), written to the host double *out -- the reduction of
 * nmg_max_dm without any device allocation.  No counterpart in the reference.
 * For callers that may not allocate GPU memory: programs whose device memory
 * belongs to their own pool, or control loops that cannot pay for the
 * device-wide synchronisation of cudaMalloc/cudaFree.  Its scratch is a fixed
 * 8 KB static device array (kept by every GPU that loads the library), which
 * limits n_nodes to 2,097,152; larger sizes return -2.  The first call on a
 * device sets that device up (make it before any stream capture); calls that
 * overlap on the GPU share the scratch and race.  Runs on the legacy default
 * stream and returns after the result is on the host; errors via
 * nmg_last_error(NULL).  The legacy stream is not ordered with non-blocking
 * streams (every handle's and batch's own stream is one), so d_m and d_m_prev
 * must be complete when the call is made: synchronise any stream that wrote
 * them first (e.g. after nmg_rhs_device or nmg_rk4_device on a handle). */
int nmg_max_dm_static(const double *d_m, const double *d_m_prev, int n_nodes, double *out);

#ifdef __cplusplus
}
#endif
#endif
