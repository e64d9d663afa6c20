/*
 * t9gb.h -- C ABI of the GB300-native AMOEBA mutual-polarization library.
 *
 * Drop-in boundary for Tinker9's induce() hot path.  Every entry point is
 * plain C: opaque context, plain pointers and sizes, int status codes, no
 * exceptions.  Each function names the reference routine it replaces
 * (paths are within the TinkerTools/tinker-gpu tree).
 *
 * Conventions
 *  - Atom arrays are in the caller's atom order; [n][3] arrays are row-major.
 *  - "_device" arrays are device pointers of the context's CUDA device; all
 *    work is issued on the context's stream (t9gb_set_stream).
 *  - Multipoles use Tinker9's MPL order: q, dx, dy, dz, qxx, qyy, qzz, qxy,
 *    qxz, qyz, in e, e*A, e*A^2 with the 1/3 quadrupole factor
 *    (include/ff/amoeba/mpole.h:4-21).
 *  - Local frames: zaxis, xaxis (0-based), yaxis (1-based, signed),
 *    kind 0 None, 1 Z-Only, 2 Z-then-X, 3 Bisector, 4 Z-Bisect, 5 3-Fold
 *    (include/ff/amoeba/mpole.h:22-36, src/elec.cpp:99-124).
 *  - Scaled pairs: rows (i, k), i < k, with scales (m, d, p, u), the union
 *    of the reference's mexclude/dpexclude/uexclude/dpuexclude tables
 *    (src/amoeba/epolar.cpp:88-484).
 */
#ifndef T9GB_H
#define T9GB_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (replace FatalError/TINKER_THROW, include/tool/error.h:15-44) */
#define T9GB_OK 0
#define T9GB_NOT_CONVERGED 1 /* PCG hit its iteration cap (src/cu/amoeba/pcg.cu:180-184) */
#define T9GB_NAN_DETECTED 2  /* non-finite residual */
#define T9GB_BAD_ARG 3
#define T9GB_CUDA_ERR 4
#define T9GB_NO_DEVICE 5
#define T9GB_NOT_READY 6 /* topology / positions / list missing */
#define T9GB_TOO_LARGE 7 /* input above a fixed capacity: atoms of the no-alloc entry point, rows of t9gb_learn_eval */

typedef struct t9gb_context t9gb_context;

/* Run-time settings.  In the reference they are Fortran module globals
 * (polpot, polpcg, ewald, pme, neigh, units); here the caller passes them. */
typedef struct {
   int n;               /* atoms */
   double box[3];       /* orthorhombic edge lengths in A; all zero: no PBC */
   int use_ewald;       /* 1: PME + Ewald real space; 0: damped Coulomb */
   double aewald;       /* Ewald coefficient, 1/A (pme.h PME::aewald) */
   int nfft[3];         /* PME grid (pme.h nfft1..3) */
   int bsorder;         /* B-spline order, must be 5 */
   double cutoff;       /* real-space cutoff, A (switchOff EWALD / MPOLE) */
   double list_buffer;  /* spatial-list buffer, A (neigh::lbuffer) */
   double usolve_cutoff;/* sparse-preconditioner cutoff, A (switchOff USOLVE) */
   double pbuffer;      /* preconditioner list buffer, A (neigh::pbuffer) */
   double poleps;       /* RMS residual threshold, Debye (polpot::poleps) */
   int politer;         /* iteration cap (polpot::politer) */
   double pcgpeek;      /* polpcg::pcgpeek */
   double udiag;        /* polpot::uaccel */
   int pcgprec;         /* 1: sparse preconditioner, 0: diagonal (polpcg::pcgprec) */
   int pcgguess;        /* 1: direct guess alpha*E, 0: zero (polpcg::pcgguess) */
   int predictor;       /* 0: none, 1: ASPC (16 frames), 2: GEAR (6) (uprior::polpred;
                           LSQR has no CUDA path in the reference: T9GB_BAD_ARG) */
   double electric;     /* kcal*A/(mol*e^2) (units::electric) */
   double debye;        /* Debye per e*A (units::debye) */
} t9gb_config;

/* Create a context on the current CUDA device.  Replaces the RcMan set-up
 * chain for this path (src/rcman.cpp:49-80: epolarData, pmeData, fftData,
 * nblistData). */
int t9gb_create(const t9gb_config* cfg, t9gb_context** out);
void t9gb_destroy(t9gb_context* ctx);
const char* t9gb_status_string(int status);
const char* t9gb_last_error(const t9gb_context* ctx);

/* Use the caller's cudaStream_t (passed as void*); NULL selects the
 * context's own stream.  Replaces g::s0 (src/cudalib.cpp:34-54). */
int t9gb_set_stream(t9gb_context* ctx, void* stream);

/* Topology, host pointers, copied once.  Replaces epolarData/mpoleData INIT
 * (src/amoeba/epolar.cpp:486-508, src/elec.cpp:91-140).
 * frames[n][4], pole[n][10] local-frame multipoles, polarity/thole/pdamp[n],
 * excl_ik[nexcl][2], excl_scale[nexcl][4] (m, d, p, u). */
int t9gb_set_topology(t9gb_context* ctx, const int* frames, const double* pole, const double* polarity,
   const double* thole, const double* pdamp, int nexcl, const int* excl_ik, const double* excl_scale);

/* Per-type-pair Thole coefficients.  ptype[n] in 0..ntypes-1 is each atom's
 * polarization type and thlval[ntypes][ntypes] (symmetric, finite, >= 0) the
 * coefficient of a pair of types, as the reference's CUDA pair kernels read
 * thlval[njpolar * jpolar[i] + jpolar[k]] (src/cu/amoeba/ufield_cu1.cc,
 * dfield_cu1.cc, sparsePrecond_cu1.cc, epolar_cu1.cc).  Replaces the jpolar /
 * thlval INIT of epolarData (src/amoeba/epolar.cpp:393-398, 486-491); Tinker
 * fills the table from the thole values and its POLPAIR keywords.
 * ntypes = 0 returns to min(thole_i, thole_k) (damp_thole2/3,
 * include/seq/damp.h:19-44).  Like t9gb_set_topology, call before
 * t9gb_nblist_build; ntypes <= 256. */
int t9gb_set_thole_pairs(t9gb_context* ctx, int ntypes, const int* ptype, const double* thlval);

/* Uniform external electric field field[3] in e/A^2 (Tinker's MV/cm value
 * divided by 1439.96455), or NULL for none.  Replaces extfld::texfld and
 * its consumers: the permanent field of both dipole sets gains the field
 * (extfieldModifyDField, src/elec.cpp:836-842, src/cu/amoeba/empole.cu:
 * 139-167), and the multipole terms gain -f (q r.E + d.E) per atom with its
 * force, torque and virial (exfieldDipole, src/elec.cpp:820-833,
 * src/cu/amoeba/empole.cu:79-137), counted in the one-body part of
 * t9gb_empole_energy.  r is the coordinate as given: the reference wraps
 * molecules into the primary cell first (bounds(), src/atom.cpp:169-176),
 * which the caller does before passing coordinates.  The polarization
 * energy includes the field through the dot product.  May change between
 * solves (a time-dependent field); takes effect in stream order. */
int t9gb_set_external_field(t9gb_context* ctx, const double* field);

/* ---- Buffered 14-7 van der Waals (the MD path around induce) ---- */

/* Per-atom van der Waals data, copied once.  Replaces the ehal INIT of
 * vdwData (src/evdw.cpp, jvdw / radmin / epsilon / ired / kred).
 * vtype[n] in 0..ntypes-1; radmin[ntypes][ntypes] (A) and
 * epsilon[ntypes][ntypes] (kcal/mol) after the combining rules, symmetric;
 * red[n] reduction factor toward parent[n] (0-based; parent = the atom
 * itself for none); scaled pairs scaled_ik[nscaled][2] with their
 * vdw-1x-scale values; the fifth-order taper starts at `taper` and ends at
 * `off` (A).  Like t9gb_set_topology, call before t9gb_nblist_build: the
 * stored neighbour list grows to cover `off`.  ntypes = 0 removes the term. */
int t9gb_set_vdw(t9gb_context* ctx, int ntypes, const int* vtype, const double* radmin, const double* epsilon,
   const double* red, const int* parent, int nscaled, const int* scaled_ik, const double* scaled_v, double taper,
   double off);

/* Buffered 14-7 energy (kcal/mol), gradient [n][3] (device, kcal/mol/A,
 * caller order) and virial (3 x 3, row-major, kcal/mol) with the calc flags.
 * Replaces void ehal(int vers) (src/ehal.cpp; src/cu/ehal.cu,
 * include/seq/pair_hal.h:52-96). */
int t9gb_ehal(t9gb_context* ctx, int vers, double* energy, float* grad_device, double* virial);

/* Bond, angle and Urey-Bradley terms.  Replaces the ebond / eangle / eurey
 * INIT of evalence (src/evalence.cpp; include/seq/bond.h, angle.h, urey.h):
 * harmonic bonds ibnd[nbond][2] with force constants bk and ideal lengths
 * bl and the global bond-cubic / bond-quartic; harmonic angles
 * iang[nangle][3] (vertex in the middle) with ak, ideal angles anat
 * (degrees) and angle_terms[4] = angle-cubic, -quartic, -pentic, -sextic;
 * Urey-Bradley pairs iury[nurey][3] (the 1-3 distance of the ends) with uk,
 * ul and urey-cubic / -quartic.  bondunit 1, angunit (pi/180)^2, ureyunit 1
 * (Tinker's defaults).  May be called any time after t9gb_create. */
int t9gb_set_valence(t9gb_context* ctx, int nbond, const int* ibnd, const double* bk, const double* bl,
   double bond_cubic, double bond_quartic, int nangle, const int* iang, const double* ak, const double* anat,
   const double* angle_terms, int nurey, const int* iury, const double* uk, const double* ul, double urey_cubic,
   double urey_quartic);

/* Valence energy, gradient [n][3] (device) and virial with the calc flags
 * (calls the coordinates set by t9gb_set_xyz_*).  Replaces void
 * evalence(int vers) for these three terms. */
int t9gb_evalence(t9gb_context* ctx, int vers, double* energy, float* grad_device, double* virial);

/* ---- Molecular dynamics ---- */

/* Start a trajectory at positions xyz[n][3] (A) with masses[n] (g/mol) and
 * velocities vel[n][3] (A/ps, NULL for zero): sets the coordinates, builds
 * the spatial order if needed and evaluates the first gradient (the
 * integrator's KickOff, src/md/integrator.cpp:186-190).  Forces are the
 * multipole + polarization terms (induce included), plus the van der Waals
 * and valence terms when set. */
int t9gb_md_init(t9gb_context* ctx, const double* xyz, const double* mass, const double* vel);

/* nsteps velocity-Verlet steps of dt ps (BasicIntegrator::dynamic with
 * nrespa 1, src/md/integrator.cpp:70-170).  thermostat 0: none (NVE);
 * 1: Bussi velocity rescaling toward kelvin with coupling time tau ps and
 * nfree degrees of freedom (<= 0: 3n - 3), variates from a generator seeded
 * by seed (bussiThermostat, src/mdpt.cpp:41-71).  Returns the last kinetic
 * energy (kcal/mol) and temperature (K) when the pointers are not NULL. */
int t9gb_md_run(t9gb_context* ctx, int nsteps, double dt_ps, int thermostat, double kelvin, double tau_ps, int nfree,
   unsigned long long seed, double* ekin, double* temperature);

/* Current positions / velocities (host, [n][3], may be NULL) and the
 * gradient at them (device [n][3], may be NULL). */
int t9gb_md_state(t9gb_context* ctx, double* xyz, double* vel, float* grad_device);

/* The current positions as float [n][3] into device memory, ordered on the
 * context's stream (no synchronisation): a caller records a trajectory
 * frame by frame without a host round trip (the reference writes archive
 * frames from host copies, src/md/misc.cpp mdsave). */
int t9gb_md_positions_device(t9gb_context* ctx, float* xyz_device);

/* Steps integrated and PCG iterations spent in them since t9gb_md_init. */
int t9gb_md_stats(t9gb_context* ctx, long long* steps, long long* pcg_iterations);

/* Coordinates [n][3].  Replace copyPosToXyz (src/atom.cpp:161-166). */
int t9gb_set_xyz_host(t9gb_context* ctx, const double* xyz);
int t9gb_set_xyz_device(t9gb_context* ctx, const float* xyz_device);

/* Coordinates from three device arrays x[n], y[n], z[n] (float), the layout
 * of the reference's `real *x, *y, *z` (include/ff/atom.h:43-45), as
 * copyPosToXyz leaves them (src/atom.cpp:161-166).  Ordered on the
 * context's stream. */
int t9gb_set_xyz_soa_device(t9gb_context* ctx, const float* x, const float* y, const float* z);

/* Build the spatial (Morton) order of the atoms from the current coordinates
 * and the scaled-partner table; the exact neighbour list is then rebuilt on
 * the device whenever coordinates change.  Replaces spatialBuild /
 * spatialUpdate (src/spatial.cpp:201-205, src/cu/spatial.cu:149-960). */
int t9gb_nblist_build(t9gb_context* ctx);

/* Local -> global multipoles with the chirality check.  Replaces mpoleInit's
 * chkpole + rotpole (src/amoeba/mpole.cpp:28-57, src/cu/amoeba/rotpole.cu:6-43). */
int t9gb_mpole_init(t9gb_context* ctx);

/* Permanent-multipole field on d and p.  Replaces
 * void dfield(real (*field)[3], real (*fieldp)[3]) (src/amoeba/field.cpp:56-63).
 * field/fieldp: [n][3] float, device. */
int t9gb_dfield(t9gb_context* ctx, float* field_device, float* fieldp_device);

/* Mutual field -T u for d and p.  Replaces
 * void ufield(const real (*uind)[3], const real (*uinp)[3], real (*field)[3],
 * real (*fieldp)[3]) (src/amoeba/field.cpp:110-117). */
int t9gb_ufield(t9gb_context* ctx, const float* uind_device, const float* uinp_device, float* field_device,
   float* fieldp_device);

/* z = M r with the sparse preconditioner.  Replaces sparsePrecondApply
 * (src/amoeba/induce.cpp:22-26, src/cu/amoeba/precond.cu:28-43). */
int t9gb_sparse_precond_apply(t9gb_context* ctx, const float* rsd_device, const float* rsdp_device,
   float* zrsd_device, float* zrsdp_device);

/* z = alpha r with the diagonal preconditioner, caller order, device
 * arrays [n][3]; rsdp and zrsdp may both be NULL (one dipole set).
 * Replaces diagPrecond (src/cu/diagprecond.cu:5-35). */
int t9gb_diag_precond_apply(t9gb_context* ctx, const float* rsd_device, const float* rsdp_device,
   float* zrsd_device, float* zrsdp_device);

/* Mutual induced dipoles by PCG.  Replaces
 * void induce(real (*uind)[3], real (*uinp)[3]) (src/amoeba/induce.cpp:108-113,
 * src/cu/amoeba/pcg.cu:14-185).  Calls dfield itself; saves the predictor
 * history like ulspredSave.  Returns T9GB_NOT_CONVERGED like the reference's
 * FatalError at the iteration cap. */
int t9gb_induce(t9gb_context* ctx, float* uind_device, float* uinp_device);

/* End-to-end form for callers with host memory: copies xyz [n][3] in, runs
 * mpole_init + induce and copies the dipoles [n][3] out (either output may be
 * NULL). */
int t9gb_induce_host(t9gb_context* ctx, const double* xyz, double* uind, double* uinp);

/* Statistics of the last induce: iterations, final RMS residual (Debye),
 * status. */
int t9gb_induce_stats(const t9gb_context* ctx, int* iterations, double* eps_debye, int* status);

/* Direct dipoles alpha*E of the last induce/dfield, [n][3] device. */
int t9gb_get_udir(t9gb_context* ctx, float* udir_device, float* udirp_device);

/* Induced dipoles of the last solve (induce, emplar, an MD step), [n][3]
 * device, e A; either pointer may be NULL. */
int t9gb_get_uind(t9gb_context* ctx, float* uind_device, float* uinp_device);

/* Permanent-multipole energy (kcal/mol) of the current coordinates and
 * rotated multipoles (call t9gb_mpole_init first): real-space (with the
 * m-scaled exclusions), reciprocal and Ewald self parts in parts[3] (may be
 * NULL).  Replaces empole(calc::energy) (src/amoeba/empole.cpp:81-138,
 * src/cu/amoeba/empole.cu, src/cu/hippo/empole.cu:195-367,
 * include/seq/emselfamoeba.h). */
int t9gb_empole_energy(t9gb_context* ctx, double* energy, double* parts);

/* Polarization energy -1/2 f sum_i u_d,i . E_p,i of the last induce (the
 * dot-product form used for calc::v0).  Replaces epolar0DotProd
 * (src/cu/amoeba/epolar.cu:14-30, called by src/amoeba/epolar.cpp:550-572). */
int t9gb_epolar_energy(t9gb_context* ctx, double* energy);

/* Calc flags of the energy/gradient entry points, the reference's calc::
 * bits (include/tool/rcman.h:105-155). */
#define T9GB_CALC_ENERGY 0x010
#define T9GB_CALC_GRAD 0x020
#define T9GB_CALC_VIRIAL 0x040

/* Permanent-multipole energy (kcal/mol) and gradient (kcal/mol/A, device
 * float [n][3], caller order, written -- not accumulated) of the current
 * coordinates and rotated multipoles (call t9gb_mpole_init first), including
 * the forces on the frame atoms from the multipole torques.  Replaces
 * empole(int vers) (src/amoeba/empole.cpp:81-138) with its torque step
 * (src/cu/amoeba/torque.cu:8-383).  vers: any of T9GB_CALC_ENERGY,
 * T9GB_CALC_GRAD, T9GB_CALC_VIRIAL; virial[9] (row-major, kcal/mol) is the
 * strain derivative dE/d(eps)_ab of the energy, symmetrised, the reference's
 * vir_em + vir_trq convention. */
int t9gb_empole(t9gb_context* ctx, int vers, double* energy, float* grad_device, double* virial);

/* Polarization: solves induce() on the current coordinates, then the energy
 * (dot-product form) and/or the gradient at the converged dipoles.  Replaces
 * epolar(int vers) (src/amoeba/epolar.cpp:550-649): epolar_cu1 /
 * epolarEwaldRecipSelf_cu1 / epolar0DotProd / torque.  Returns the induce
 * status (T9GB_NOT_CONVERGED ...) when the solve fails. */
int t9gb_epolar(t9gb_context* ctx, int vers, double* energy, float* grad_device, double* virial);

/* Both terms in one pass over the pair list (the MD path), energy = empole +
 * epolar.  Replaces emplar(int vers) (src/amoeba/emplar.cpp:10-28,
 * src/cu/amoeba/emplar.cu:505-606). */
int t9gb_emplar(t9gb_context* ctx, int vers, double* energy, float* grad_device, double* virial);

/* A gradient [n][3] (device float, kcal/mol/A, as t9gb_empole / epolar /
 * emplar / ehal / evalence write it) into the reference's fixed-point
 * gradient arrays gx[n], gy[n], gz[n] (device, unsigned 64-bit at 2^32 per
 * kcal/mol/A, grad_prec under TINKER_DETERMINISTIC_FORCE,
 * include/ff/precision.h:102-106), converted as floatTo<fixed> does
 * (include/syntax/cu/adddef.h:36-71).  accumulate = 0 writes, 1 adds like
 * sumGradient (src/cu/egvop.cu:6-19); grad_device = NULL with accumulate = 0
 * clears the three arrays.  One word per thread: deterministic. */
int t9gb_gradient_fixed(t9gb_context* ctx, const float* grad_device, int accumulate, unsigned long long* gx_device,
   unsigned long long* gy_device, unsigned long long* gz_device);

/* Components of the last energy evaluation (t9gb_empole_energy, t9gb_empole,
 * t9gb_epolar, t9gb_emplar with T9GB_CALC_ENERGY): parts[4] = multipole
 * real-space, reciprocal and self energy, polarization energy (kcal/mol),
 * the reference's separate em/ep accumulators (src/amoeba/empole.cpp,
 * src/amoeba/epolar.cpp). */
int t9gb_energy_components(t9gb_context* ctx, double* parts);

/* Run induce() as one CUDA graph (default, enable = 1: neighbour list,
 * permanent field, guess and the PCG loop as a conditional WHILE node with
 * the convergence test on the device) or as individually launched kernels
 * with one host synchronisation per iteration (enable = 0, the reference's
 * pattern, pcg.cu:144-145).  Both give bit-identical dipoles. */
int t9gb_use_graph(t9gb_context* ctx, int enable);

/* PME 3-D FFT: the library's fused transform (enable = 1; cubic grids of 32,
 * 64 or 128 points per edge: a 2-D FFT of each z plane that also reads and
 * clears the fixed-point grid, a z-line pass that applies the influence
 * function between the forward and inverse transforms, and an inverse 2-D
 * plane pass) or cuFFT C2C plus separate conversion and convolution kernels
 * (enable = 0; always used for other grid sizes).  The default is the fused
 * transform on 32^3 and 64^3 grids, where it measured faster on GB300, and
 * cuFFT on every other grid, 128^3 included.  Replaces fftfront/fftback +
 * pmeConv (src/cudart/fft.cpp:65-95, src/cu/pme.cu:908-1031).  Enabling on
 * an unsupported grid returns T9GB_BAD_ARG. */
int t9gb_pme_own_fft(t9gb_context* ctx, int enable);

/* Partition of the fused transform's two plane passes: ctas = 0 (the
 * default) runs one CTA per z plane; 2, 4 or 8 (8 on grids of 64 points
 * per edge or more) spread each plane over a thread-block cluster of that
 * many CTAs, which stage their row slabs with bulk asynchronous copies and
 * exchange rows for columns through distributed shared memory.
 * Bit-identical results either way.  A tuning knob: on GB300 at 64^3 the
 * clustered passes measured 22.8 / 24.2 / 25.0 us per transform +
 * convolution against 21.0 us for one CTA per plane. */
int t9gb_pme_fft_cluster(t9gb_context* ctx, int ctas);

/* Staged real-space mutual-field and preconditioner kernels (enable = 1):
 * each 32-atom block copies the rows of the neighbouring 32-atom blocks it
 * needs into shared memory with bulk asynchronous copies and reads every
 * neighbour from there; enable = 0 (the default) reads each neighbour row
 * from global memory through L1.  Bit-identical fields either way (the same
 * pairs in the same order); used with 4 or 8 lanes per atom.  A tuning knob:
 * measured on GB300 the staged kernels are slower (mutual field 22.6 vs
 * 20.7 us at 12,288 atoms, 161 vs 101 us at 98,304), because a block stages
 * about 39 neighbouring blocks of 1.5 KB, three times the rows it reads,
 * while the global kernels hit L1 on 85% of their row sectors. */
int t9gb_pair_staging(t9gb_context* ctx, int enable);

/* Device flags of the library's asynchronous copies, read after a
 * synchronisation: bit 0 a staging copy of the pair kernels, bit 1 a slab
 * copy of the transform's clustered plane passes, bit 2 a tensor-core
 * product of the learned-guess network did not complete within the
 * kernel's bounded wait (the kernel then went on and its results are not
 * valid).  Zero in normal operation. */
int t9gb_copy_error(t9gb_context* ctx, int* flag);

/* Lanes of a warp that share one atom's neighbour row in the real-space
 * field and preconditioner kernels: 4, 8, 16 or 32 (default 8 up to 32,768
 * atoms, 4 above).  A tuning knob; results are identical up to the order of
 * the per-lane partial sums. */
int t9gb_pair_lanes(t9gb_context* ctx, int lanes);

/* Lanes of a warp that share one atom's neighbour row in the real-space
 * force kernel (empole / epolar / emplar gradients): 4 (default), 8 or
 * 16.  A tuning knob; results are identical up to the order of the
 * per-lane partial sums.  Measured on GB300 (emplar gradient, 12,288 /
 * 98,304 atoms, ms): 1 lane 0.817 / 4.031, 2 0.781 / 4.051, 4 0.758 /
 * 4.071, 8 0.768 / 4.148, 16 0.797 / 4.355 (1 and 2 are not built). */
int t9gb_force_lanes(t9gb_context* ctx, int lanes);

/* Kernel fusion and overlap of the CG solve (bit mask; default 121 = 64 | 32 | 16 | 8 | 1).  Bit 0: the
 * sparse preconditioner also forms r.z, r.r and the CG scalars (else a
 * separate dot kernel, sparsePrecondApply + the dot products of
 * src/cu/amoeba/pcg.cu:120-150).  Bit 1 (PME only): the search direction
 * p = z + b p is formed by the kernels that read it (spread, real-space
 * field, gather, and the Ap kernel, which stores it) instead of by a
 * kernel of its own.  Bit 2 (with bit 1): the gather also forms Ap, p.Ap
 * and the step length.  Bit 3 (PME with a predictor): once the predictor's
 * ring is full the field of the extrapolated guess is computed beside the
 * permanent field (the guess does not depend on it), on the second grid and
 * two more streams, with the same kernels and sums as in order.  Bit 4: the
 * kernels of the PCG loop (search direction, spread, transform passes,
 * real-space field, gather, Ap, update, preconditioner) are launched as
 * programmatic dependents of the kernel before them on their stream: each
 * is scheduled while its predecessor drains and waits for it at its start
 * (griddepcontrol), which gives the same results as plain launches; GB300:
 * 0.527 -> 0.514 ms at 12,288 atoms, 2.313 -> 2.293 ms at 98,304.  Bit 5
 * (PME, without bit 1): the search direction's gather runs right after the
 * transform on the reciprocal stream, as a programmatic dependent of its
 * last pass (the spread and the gather form their B-splines, which need
 * the positions only, before they wait), and stores recip + self apart; the
 * Ap kernel adds it to the real-space field, the sum the gather would form.
 * Bit 6 (with bit 5): that chain stays on the main stream behind the
 * direction kernel and the real-space field runs on the side stream.  Bits
 * 5-6 give the same bits as without them; GB300 (induce ms, 12,288 /
 * 98,304 atoms): mask 25 0.4925 / 2.344, 57 0.4829 / 2.297, 121 (the
 * default) 0.473 / 2.285.  A tuning knob: the same iteration, results equal
 * up to the order of the partial sums.  Measured on GB300 (induce ms per
 * step, 12,288 / 98,304 atoms): mask 0 0.612 / 2.889, 1 0.609 / 2.853,
 * 3 0.606 / 2.959, 7 0.632 / 2.962.  Bit 1 makes the real-space kernel read
 * two rows per neighbour, which costs where that kernel is the longer arm
 * of the iteration; bit 2 makes the gather hold more registers and hide
 * less of its grid-load latency. */
int t9gb_set_pcg_fusion(t9gb_context* ctx, int mask);

/* Neighbour-list sizes: row capacity, entries of the current list (both
 * directions) and scaled pairs (the reference's Spatial::nakpl/niak,
 * include/ff/spatial.h:15-140). */
int t9gb_nblist_stats(t9gb_context* ctx, int* capacity, long long* entries, int* nscaled);

/* Mutual field without any allocation.  No counterpart in the reference: it
 * is for callers that may not call cudaMalloc when they need the field --
 * hosts that own every device allocation, code running inside a CUDA-graph
 * stream capture, real-time loops that forbid allocator calls after
 * start-up.  Inputs and outputs are the caller's device arrays (xyz, uind,
 * uinp, field, fieldp [n][3]; pdamp, thole [n]); the working memory is a
 * static device array inside the library sized for
 * T9GB_NOALLOC_MAX_ATOMS atoms (384 KiB, held by every GPU that loads the
 * library until the process exits).  It computes the damped (non-Ewald)
 * field -T u of pairs within `cutoff` (minimum image when box != NULL has
 * three positive edges), all mutual scales 1, like t9gb_ufield on a context
 * with use_ewald = 0.  n > T9GB_NOALLOC_MAX_ATOMS returns T9GB_TOO_LARGE.
 * The first call on each device looks up the array's address
 * (cudaGetSymbolAddress) and should therefore happen before any stream
 * capture.  Every call reuses the same array: calls that can overlap on the
 * GPU (different streams, no ordering between them) race. */
#define T9GB_NOALLOC_MAX_ATOMS 8192
int t9gb_ufield_noalloc(int n, const double* box, double cutoff, const float* xyz_device, const float* pdamp_device,
   const float* thole_device, const float* uind_device, const float* uinp_device, float* field_device,
   float* fieldp_device, void* stream);

/* Learned initial guess.  No counterpart in the reference, whose guesses are
 * alpha*E (src/cu/amoeba/induce.cu pcgUdirV2) and the ASPC/GEAR/LSQR
 * predictors (src/amoeba/induce.cpp:29-69).  A per-atom network
 * 32 -> 64 SiLU -> 64 SiLU -> 3 (BF16 weights and activations, FP32
 * accumulation, tensor-core GEMMs) maps rotation-invariant features of each
 * atom -- its direct field E and polarizability, radial/charge/polarizability
 * Gaussian descriptors and the first-order mutual field of the neighbours'
 * direct dipoles within 6 A, all in the atom's local multipole frame -- to a
 * correction of alpha*E.  mode bit 0: after each solve, one AdamW step
 * (learning rate lr, decoupled weight decay) on the converged dipoles of that
 * solve; bit 1: start each PCG solve (d and p separately) from the learned
 * guess when its residual r.r is smaller than that of the plain guess
 * (the predictor's when its history is full).  The PCG convergence test is
 * unchanged.  Both bits run inside the induce() graph. */
#define T9GB_LEARN_NFEAT 32
#define T9GB_LEARN_NPARAM 6792 /* W1[32][64] b1[64] W2[64][64] b2[64] W3[64][8] b3[8] (cols 3-7 of W3, b3 unused) */
int t9gb_learn_config(t9gb_context* ctx, int mode, double lr, double weight_decay);
/* Fresh Glorot-uniform weights from `seed`; clears the optimiser moments, the
 * frozen feature statistics and the target scale. */
int t9gb_learn_reset(t9gb_context* ctx, unsigned seed);
/* How often both starts are compared (bit 1 of the mode).  probe_every = 1
 * (default): every solve computes both starting residuals and picks per
 * system.  probe_every = k > 1: the comparison runs on every k-th solve, when
 * the predictor history has just filled and whenever the last comparison
 * split d and p; the solves in between start from what it chose for both
 * systems, so they pay for one starting residual only. */
int t9gb_learn_policy(t9gb_context* ctx, int probe_every);
/* Last solve: choice bit 0 / 1 = the d / p solve started from the learned
 * guess; starting RMS residuals (Debye, the PCG's definition) of the plain and
 * the learned guess at the last comparison; training loss (mean squared error
 * in target-scale units); compared = 1 when this solve ran the comparison. */
int t9gb_learn_stats(t9gb_context* ctx, int* choice, double* eps0_plain, double* eps0_learned, double* loss,
   int* compared);
int t9gb_learn_get_weights(t9gb_context* ctx, float* w, int nparam);
int t9gb_learn_set_weights(t9gb_context* ctx, const float* w, int nparam);
/* Network forward and backward on caller rows, host arrays: x[rows][32]
 * (rounded to BF16), targets t[rows][3] -> y[rows][3], grad[T9GB_LEARN_NPARAM]
 * of the loss mean((y - t)^2), and the loss.  For gradient checks; rows at
 * most 2 x the atom count rounded up to 32 (else T9GB_TOO_LARGE). */
int t9gb_learn_eval(t9gb_context* ctx, int rows, const float* x, const float* t, float* y, float* grad,
   double* loss);
/* One AdamW step (beta 0.9/0.999, eps 1e-8) with the gradient of the last
 * t9gb_learn_eval. */
int t9gb_learn_adamw(t9gb_context* ctx);
/* Tensor-core path of the network: 1 (default) the fifth-generation tensor
 * cores (tcgen05.mma, accumulators in tensor memory): one fused kernel per
 * 128 rows for the forward pass, and for training one persistent kernel
 * that recomputes the forward pass and accumulates the weight gradients in
 * tensor memory, then one kernel for the fixed-order gradient sum and the
 * AdamW step; 0 the warp-level mma.sync GEMMs with separate bias, SiLU,
 * loss, column-sum and AdamW kernels.  Same rounding points (gradients
 * within 1.2e-7 relative in the tests).  GB300, 12,288 atoms: a training
 * solve 1.045 (path 0) -> 0.860 ms (plain 0.789 ms). */
int t9gb_learn_tensor_path(t9gb_context* ctx, int path);

/* Learned extrapolation of the predictor ring (ASPC or Gear contexts): after
 * every solve, a least-squares fit of the converged dipoles on the `order`
 * most recent ring frames (2 .. 8 with ASPC's ring of 16, 2 .. 5 with Gear's
 * ring of 6; their backward differences as the basis, normal equations over
 * every element of both dipole sets kept in FP64 with forgetting factor 0.99,
 * solved on the device) gives the ring coefficients of the next solve's
 * start, in place of the predictor's (from the second fit on).  The PCG
 * convergence test is unchanged.  0 (the default) keeps the predictor's own
 * coefficients.  Every call starts a new fit.  T9GB_BAD_ARG for other
 * orders or without a predictor. */
int t9gb_learn_extrapolation(t9gb_context* ctx, int order);
/* State of the learned extrapolation after the last solve: the fits so far
 * (*fits), those whose solve failed and left the previous coefficients in
 * place (*rejected), and the 16 ring coefficients by frame age (coef[0] the
 * newest frame; 0 beyond the order).  Zeros while the extrapolation is off. */
int t9gb_learn_extrapolation_state(t9gb_context* ctx, int* fits, int* rejected, float* coef16);
/* Raw features of the last solve, device [2n][32]: rows 0..n-1 for the d
 * dipoles, n..2n-1 for the p dipoles, caller atom order. */
int t9gb_learn_features(t9gb_context* ctx, float* features_device);

/* Tracing: per-kernel CUDA-event timing of every launch of the listed
 * categories (the reference has only cudaProfilerStart/Stop,
 * src/cudalib.cpp:20,53).  Enabling allocates the event pool; reading
 * returns the accumulated milliseconds and launch count of one category and
 * reset != 0 clears them. */
#define T9GB_PROF_NCAT 10
int t9gb_profile_enable(t9gb_context* ctx, int enable);
int t9gb_profile_read(t9gb_context* ctx, int category, double* total_ms, long long* launches, int reset);
const char* t9gb_profile_name(int category);

#ifdef __cplusplus
}
#endif
#endif
