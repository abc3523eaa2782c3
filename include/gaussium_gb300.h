/*
 * gaussium_gb300 -- C ABI of the GB300 (sm_103a) two-electron-integral and Fock-build
 * engine.  The reference Gaussium is pure Python and has no FFI; these entry points are
 * what its ERI path binds through ctypes (the Python package gaussium_gb300 is that
 * binding).  Each one cites the reference function it replaces (file:line within the
 * reference project).
 *
 * Conventions
 *   - All array arguments are DEVICE pointers owned by the caller (torch tensors in the
 *     Python host code); `stream` is a cudaStream_t passed as void*.  No entry point
 *     allocates device memory.
 *   - Every entry point returns a status code: 0 = GS_OK, otherwise one of GS_ERR_*;
 *     gs_status_string() gives its text.  Nothing throws or aborts across the ABI.
 *   - Launches are asynchronous on `stream`; errors of the kernels themselves surface at
 *     the caller's next synchronisation.
 *   - Records (sizes from gs_record_sizes):
 *       PairRec  48 B  {double AB[3]; int prim_off, nprim, sa, sb; float qmax; int pad;}
 *       Prim64   80 B  {double p, 1/(2p), P[3], PA[3], Kp, pad;}   pad = first shell's exponent
 *       Prim32   48 B  {float  p, 1/(2p), P[3], PA[3], Kp, pad[3];}   pad[0] = the same
 *       WriteTask 24 B {int bra, ket, code, pad; long long off;}
 *   - Shells: l <= 2, Cartesian components in the reference order
 *     (s; x,y,z; xx,yy,zz,xy,xz,yz -- factory/primitive_basis_factory.py:5-86), effective
 *     contraction coefficients and per-component scale factors as built by
 *     gaussium_gb300/basis.py from the reference's normalisations
 *     (objects/basis_function.py:22-53, objects/primitive_basis_function.py:26-42).
 */
#ifndef GAUSSIUM_GB300_H
#define GAUSSIUM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define GS_OK 0
#define GS_ERR_ARG 1
#define GS_ERR_CUDA 2
#define GS_ERR_CLASS 3
#define GS_ERR_DEVICE 4
#define GS_ERR_NOMEM 5
#define GS_ERR_LIMIT 6

/* Library version (1). */
int gs_version(void);

/* Text of a status code (static storage). */
const char* gs_status_string(int status);

/* sizes[0..3] = sizeof PairRec, Prim64, Prim32, WriteTask (host pointer). */
int gs_record_sizes(int* sizes);

/* 1 if the (la lb | lc ld) class kernel is built into this library, else 0. */
int gs_class_available(int la, int lb, int lc, int ld);

/* Kernel forms built for class (la lb|lc ld) in the given precision (64 or 32): bit 0 the
 * one-thread-per-quartet kernel, bit 1 the warp-per-quartet kernel, bit 2 the warp kernel
 * that runs several primitive quartets through each recursion pass, bit 3 the split form
 * (the thread kernel's code, one warp per quartet over its primitive quartets), bit 4 the
 * cooperative form (the warp kernel's code, up to eight warps per quartet), bit 5 the
 * stacked form (the warp kernel with each lane's node record run on several primitive
 * quartets: 2 in FP64, 4 in FP32); negative status on a bad class or precision.  No
 * reference counterpart (the reference has one code path). */
int gs_class_variants(int la, int lb, int lc, int ld, int precision);

/* Chooses the kernel form later calls use for (la lb|lc ld) in that precision, process-wide:
 * 0 = the built-in default by total angular momentum, 1 = thread per quartet, 2 = warp per
 * quartet, 3 = grouped warp per quartet, 4 = split, 6 = stacked warp per quartet (a form
 * the class was not built with, or the per-call cooperative form 5, is GS_ERR_ARG).
 * Results do not depend on the form beyond rounding; the autotuner times the forms on the
 * caller's task lists.  No reference counterpart. */
int gs_set_class_variant(int la, int lb, int lc, int ld, int precision, int variant);

/* The kernel form (1 thread, 2 warp, 3 grouped warp, 4 split, 6 stacked) a launch of
 * (la lb|lc ld) in that precision uses with no explicit form: the configured variant, or
 * the built-in default.
 * The precision argument of gs_eri_blocks, gs_fock_jk and gs_fock_jk_batched may carry an
 * explicit form in its bits 8.. (precision | form << 8, forms 1-6 as gs_class_variants'
 * bits 0-5) for that call only; the engine uses it to run the quartets with many primitive
 * quartets (the heavy prefix of a class's task list, sorted by descending primitive work)
 * in the split form where the class runs one thread per quartet, and in the cooperative
 * form where it runs one warp per quartet (warp, grouped or stacked).  The cooperative form
 * takes host task counts only.  Negative status on a bad class or precision.  No reference counterpart. */
int gs_class_form(int la, int lb, int lc, int ld, int precision);

/* K0 shell-pair builder.  Replaces the per-primitive-quartet prologue of
 * ObaraSaika.integrate (integrals/twoelectronrepulsion/obara_saika_scheme.py:52-70:
 * Gaussian product centre, exponent sums, exp(-ab/p |AB|^2) and the contraction/
 * normalisation product), hoisted to once per primitive *pair*.
 * Shells: centre[nshell*3] (bohr), l[nshell], prim_off[nshell+1], expo[nprim],
 * coef[nprim].  Pairs: pair_shells[npairs*2] (l[first] >= l[second]),
 * pair_prim_off[npairs] (first primitive-pair record of each pair, Ka*Kb reserved).
 * Outputs: pair_rec[npairs], prim64, prim32 (may be NULL), kept[npairs] (may be NULL:
 * primitive pairs kept).  max_exp > 0 drops primitive pairs with
 * alpha*beta/(alpha+beta)*|AB|^2 > max_exp (0 keeps all, as the reference does).
 * group_start[ngroups+1] (device; ngroups 0 = one warp per pair) packs consecutive pairs
 * into groups whose primitive pairs (Ka*Kb each) total at most 32, or single pairs:
 * one warp per group keeps its lanes busy on small pairs. */
int gs_pairs_build(const double* centre, const int* l, const int* prim_off, const double* expo,
                   const double* coef, int npairs, const int* pair_shells,
                   const int* pair_prim_off, void* pair_rec, void* prim64, void* prim32,
                   double max_exp, int* kept, int ngroups, const int* group_start,
                   void* stream);

/* K1 Schwarz bounds q[p] = sqrt(max |(ab|ab)|) for the npair pairs pair_index[] of class
 * (la lb), in FP64; then copies all npairs_total bounds into pair_rec[].qmax.  No
 * reference counterpart (the reference does not screen); it feeds the screened quartet
 * lists that stand in for the key loop of create_repulsion_matrix
 * (matrixelements/electron_repulsion_matrix.py:30-33). */
int gs_schwarz(int la, int lb, void* pair_rec, const void* prim64, const double* comp_scale,
               int npair, const int* pair_index, double* q, int npairs_total, void* stream);

/* K3 ERI class kernel, block output.  Replaces ObaraSaika.integrate /
 * HeadGordonPople.integrate / ElectronRepulsion.integrate
 * (obara_saika_scheme.py:17-82, head_gordon_pople.py:18-91, cook_integral.py:15-99) for
 * every function quartet of ntask shell quartets of class (la lb | lc ld) at once
 * (la >= lb, lc >= ld, bra pair class >= ket pair class).  tasks[] are WriteTasks; block
 * q is written to out + off in the caller's original (a,b,c,d) order, row-major.
 * precision 64: FP64 throughout; 32: FP32 evaluation, FP64 output. */
int gs_eri_blocks(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
                  const void* prim, const double* comp_scale, int ntask, const void* tasks,
                  double* out, void* stream);

/* K3+K4 integral-direct Coulomb/exchange digestion.  Replaces the Python element loops
 * of FockMatrixRestricted.create (hartreefock/fock_matrix.py:12-22),
 * FockMatrixUnrestricted.create (fock_matrix.py:32-53),
 * BlockedFockMatrixUnrestricted.create (fock_matrix.py:63-81) and the Coulomb part of
 * RestrictedKohnShamHamiltonian.create (kohnsham/kohn_sham_hamiltonian.py:15-19),
 * which read a stored N^4 tensor.  For the ntask unique shell quartets tasks[2*t] =
 * (bra pair, ket pair) of class (la lb | lc ld) it accumulates (FP64 atomics)
 *   J'_ab += 2 v P_cd, J'_cd += 2 v P_ab                  (if pj and j are given)
 *   K'_ac += v P_bd, K'_ad += v P_bc, K'_bc += v P_ad, K'_bd += v P_ac   (nk densities)
 * with v the quartet's integral over its permutation multiplicity; the caller forms
 * J = J' + J'^T and K = K' + K'^T.  Matrices are nbf x nbf row-major.  With
 * screen_thr > 0 a quartet is evaluated only if qmax_bra*qmax_ket*max|P| over its six
 * shell blocks (shell_dmax[nshell*nshell]) is >= screen_thr and lies in
 * [prec_lo, prec_hi) -- the mixed-precision split.  precision 64 or 32 (FP32 integrals
 * and digestion, FP64 accumulation). */
int gs_fock_jk(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
               const void* prim, const double* comp_scale, const int* func_off, int nshell,
               int nbf, int ntask, const int* tasks, const double* pj, double* j, int nk,
               const double* pk, double* k, const double* shell_dmax, double screen_thr,
               double prec_lo, double prec_hi, void* stream);

/* Bytes of device workspace gs_fock_jk_mixed needs for ntask tasks. */
long long gs_fock_jk_mixed_workspace(int ntask);

/* Mixed-precision form of gs_fock_jk (same replaced reference functions).  A partition
 * kernel splits the ntask tasks by est = qmax_bra qmax_ket max|P| (over the quartet's six
 * shell blocks, shell_dmax[nshell*nshell]): est >= mixed_cut -> FP64 (prim64 records),
 * screen_thr <= est < mixed_cut -> FP32 (prim32 records), est < screen_thr -> skipped; the
 * two lists and their counts live in the caller's workspace (ws_bytes >=
 * gs_fock_jk_mixed_workspace(ntask)), and the two class launches read their counts there,
 * so the call needs no host synchronisation.  Accumulation is FP64 in both cases. */
int gs_fock_jk_mixed(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                     const void* prim32, const double* comp_scale, const int* func_off,
                     int nshell, int nbf, int ntask, const int* tasks, const double* pj, double* j,
                     int nk, const double* pk, double* k, const double* shell_dmax,
                     double screen_thr, double mixed_cut, void* workspace, long long ws_bytes,
                     void* stream);

/* gs_fock_jk_mixed without a workspace argument, for callers that cannot allocate device
 * memory: a host whose memory manager owns every device allocation and forbids further
 * ones, or a C/C++ caller with no device allocator of its own.  It makes no cudaMalloc,
 * cudaFree or other allocating call.  Its scratch (the two partitioned task lists and
 * their counts) lives in one fixed array of 16 MiB + 256 B in device memory, held by
 * every GPU that loads the library until the process exits; ntask above
 * gs_fock_jk_mixed_noalloc_max_tasks() (2^20) returns GS_ERR_LIMIT.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current, so make that first call before any stream capture.  The address is kept for
 * the life of the process: after cudaDeviceReset (or anything else that re-creates the
 * device's primary context) the kept address is stale, so do not call this entry point
 * again in that process.  All calls share the one
 * array: the counts are cleared at the start of every call, and calls that overlap on
 * the GPU (different streams, no ordering) race.  No counterpart in the reference. */
int gs_fock_jk_mixed_noalloc(int la, int lb, int lc, int ld, const void* pair_rec,
                             const void* prim64, const void* prim32, const double* comp_scale,
                             const int* func_off, int nshell, int nbf, int ntask, const int* tasks,
                             const double* pj, double* j, int nk, const double* pk, double* k,
                             const double* shell_dmax, double screen_thr, double mixed_cut,
                             void* stream);

/* Largest ntask gs_fock_jk_mixed_noalloc accepts (2^20). */
int gs_fock_jk_mixed_noalloc_max_tasks(void);

/* Batched form of gs_fock_jk for many molecules in one launch (the reference builds one
 * molecule at a time; same replaced functions as gs_fock_jk).  shell_mol[s] is the
 * molecule of shell s; molecule m's nbf_m x nbf_m matrices start at mol_base[m] in pj, j, pk
 * and k, with nbf_m = mol_n[m]; func_off is local to each molecule.  nk <= 1 exchange
 * density; mat_stride is the element count of one full set of matrices.  With
 * screen_thr > 0 the density factor of the screening bound is mol_dmax[m]. */
int gs_fock_jk_batched(int la, int lb, int lc, int ld, int precision, const void* pair_rec,
                       const void* prim, const double* comp_scale, const int* func_off,
                       const int* shell_mol, const long long* mol_base, const int* mol_n,
                       const double* mol_dmax, long long mat_stride, int ntask, const int* tasks,
                       const double* pj, double* j, int nk, const double* pk, double* k,
                       double screen_thr, double prec_lo, double prec_hi, void* stream);

/* Mixed-precision, density-screened form of gs_fock_jk_batched: a partition kernel splits
 * the tasks by est = qmax_bra qmax_ket dmax into an FP64 list (est >= mixed_cut), an FP32
 * list (screen_thr <= est < mixed_cut) and dropped tasks, in the caller's workspace
 * (ws_bytes >= gs_fock_jk_mixed_workspace(ntask)); the class launches read the list lengths
 * on the device and stride over them, so a batch whose densities barely change
 * (incremental builds near convergence) costs little more than the partition.  dmax is the
 * largest |P| over the six shell blocks of the quartet, from molecule m's own block table
 * at mol_dmax + mol_sbase[m] (mol_nshell[m] x mol_nshell[m], shells numbered from
 * mol_shell0[m]); with those three arrays null, mol_dmax[m] is one value per molecule.
 * Same replaced reference functions as gs_fock_jk. */
int gs_fock_jk_batched_mixed(int la, int lb, int lc, int ld, const void* pair_rec,
                             const void* prim64, const void* prim32, const double* comp_scale,
                             const int* func_off, const int* shell_mol, const long long* mol_base,
                             const int* mol_n, const double* mol_dmax, const int* mol_shell0,
                             const int* mol_nshell, const long long* mol_sbase,
                             long long mat_stride, int ntask, const int* tasks, const double* pj,
                             double* j, int nk, const double* pk, double* k, double screen_thr,
                             double mixed_cut, void* workspace, long long ws_bytes, void* stream);

/* K2 Boys function F_0..F_m(t) (m <= 10) of n arguments t[] into F[n*(m+1)], in FP64 or
 * FP32 (results widened to FP64).  Replaces boys_function / boys_function_recursion
 * (integrals/boys_function.py:4-76). */
int gs_boys_eval(int m, int precision, int n, const double* t, double* F, void* stream);

/* K7 one-electron integrals over npairs shell pairs pair_shells[2*p] (any order of l; each
 * unordered pair once): overlap S, kinetic T (-1/2 nabla^2 on the ket) and nuclear
 * attraction V of natom point charges atom_z[] at atom_xyz[3*natom], written to both (a,b)
 * and (b,a) blocks of the nbf x nbf matrices (V is zeroed first and summed over the nuclei,
 * one thread per pair and nucleus).  Replaces OrbitalOverlapMatrix / KineticEnergyMatrix /
 * NuclearAttractionMatrix .create (matrixelements/orbital_overlap_matrix.py:15-27,
 * kinetic_energy_matrix.py:16-33, nuclear_attraction_matrix.py:16-29) and the integrals
 * they call (integrals/orbital_overlap_integral.py:16-36,
 * integrals/nuclear_attraction_integral.py:19-57). */
int gs_one_electron(const double* centre, const int* l, const int* prim_off, const double* expo,
                    const double* coef, const double* comp_scale, const int* func_off,
                    int npairs, const int* pair_shells, int nbf, int natom,
                    const double* atom_xyz, const double* atom_z, double* S, double* T,
                    double* V, void* stream);

/* K6 ERI adjoint.  For nq unique shell quartets quartets[4*q] = (A,B,C,D) it contracts the
 * derivative integrals with the RHF weights
 *   Gamma_abcd = w (1/2 P_ab P_cd - 1/8 (P_ac P_bd + P_ad P_bc)),  w = orbit size,
 * and adds dE/dR into grad[natom*3] (FP64 atomics) through shell_atom[] (D by
 * translational invariance).  block_off[6*q + 2*c] / [6*q + 2*c + 1] give the offsets in
 * blocks[] of the raised / lowered block of centre c (A, B, C) in (A,B,C,D) order (-1 if
 * absent), as written by gs_eri_blocks for the raised shell (l+1, coefficients times
 * 2 alpha, unit component scales) and the lowered shell (l-1).  No reference counterpart:
 * the reference has no gradients and optimises with Nelder-Mead
 * (geometryoptimization/nelder_mead.py:28-144). */
int gs_eri_grad_contract(int nq, const int* quartets, const long long* block_off,
                         const double* blocks, const int* l, const int* func_off,
                         const double* comp_scale, const int* shell_atom, int nbf,
                         const double* density, double* grad, void* stream);

/* K6 fused ERI adjoint for the s/p/d classes (la lb | lc ld) (l <= 2, la >= lb, lc >= ld,
 * (la,lb) >= (lc,ld)): for the ntask unique quartets tasks[2*t] = (bra pair, ket pair) it
 * evaluates the derivative integrals of centres A, B, C in one pass (VRR per primitive
 * quartet into four weighted contraction sets 1, 2 alpha, 2 beta, 2 gamma, up to l + 1 on
 * the differentiated centre; six HRR blocks in shared memory), contracts them, times the
 * component scales of all four functions, with the same RHF weights as
 * gs_eri_grad_contract and adds dE/dR to grad[natom*3] through shell_atom[] (every entry
 * in [0, natom)).  prim64 records must carry the first shell's exponent in their pad
 * field (gs_pairs_build writes it).  No reference counterpart (see gs_eri_grad_contract). */
int gs_eri_grad(int la, int lb, int lc, int ld, const void* pair_rec, const void* prim64,
                const double* comp_scale, const int* func_off, const int* shell_atom, int ntask,
                const int* tasks, int nbf, int natom, const double* density, double* grad,
                void* stream);

/* gs_eri_grad with an explicit kernel form for this call: 0 = the class's configured form,
 * 1 = one thread per quartet, 2 = one warp per quartet, 3 = split (the thread code with one
 * warp per quartet over its primitive quartets, for quartets with many of them); forms 1
 * and 3 exist for classes of total angular momentum <= 3 (else GS_ERR_ARG).  No reference
 * counterpart (see gs_eri_grad_contract). */
int gs_eri_grad_form(int la, int lb, int lc, int ld, int form, const void* pair_rec,
                     const void* prim64, const double* comp_scale, const int* func_off,
                     const int* shell_atom, int ntask, const int* tasks, int nbf, int natom,
                     const double* density, double* grad, void* stream);

/* gs_eri_grad_form restricted to a band of the density-weighted bound, in a chosen
 * precision: a quartet is evaluated when q_ab q_cd max|P| over its six shell blocks
 * (shell_dmax, nshell x nshell, device) is at least screen_thr and in [prec_lo, prec_hi)
 * (screen_thr <= 0: every quartet).  precision 32 evaluates the recursion and the weighted
 * contraction in FP32 from FP32 records (thread and split forms only; the Boys function
 * below its asymptotic threshold stays FP64), the HRR, contraction with the density and
 * the gradient sums in FP64.  No reference counterpart (see gs_eri_grad_contract). */
int gs_eri_grad_band(int la, int lb, int lc, int ld, int form, int precision,
                     const void* pair_rec, const void* prim, const double* comp_scale,
                     const int* func_off, const int* shell_atom, int ntask, const int* tasks,
                     int nbf, int natom, const double* density, int nshell,
                     const double* shell_dmax, double screen_thr, double prec_lo,
                     double prec_hi, double* grad, void* stream);

/* The form (1 thread, 2 warp) a gs_eri_grad launch of that class uses: the configured
 * variant or the default; negative status on a class without gradient kernels.  No
 * reference counterpart. */
int gs_eri_grad_class_form(int la, int lb, int lc, int ld);

/* Kernel forms built for gradient class (la lb|lc ld): bit 0 one thread per quartet
 * (classes of total angular momentum <= 3), bit 1 one warp per quartet; negative status
 * for a class without gradient kernels.  No reference counterpart. */
int gs_eri_grad_variants(int la, int lb, int lc, int ld);

/* Chooses the form later gs_eri_grad calls use for that class, process-wide: 0 = default
 * (thread per quartet up to total angular momentum 2, warp above), 1 = thread, 2 = warp.
 * No reference counterpart. */
int gs_set_eri_grad_variant(int la, int lb, int lc, int ld, int variant);

/* One-electron part of the RHF gradient: for npairs unique shell pairs (a >= b) adds
 *   f sum_ij [P_ij (dT_ij + dV_ij) - W_ij dS_ij]   (f = 2 for a != b, 1 for a == b)
 * to grad[natom*3] through shell_atom[], including the nuclear-attraction operator term
 * of every nucleus.  density P and energy_weighted W are nbf x nbf.  No reference
 * counterpart (the reference has no gradients); it differentiates the integrals of
 * integrals/orbital_overlap_integral.py, matrixelements/kinetic_energy_matrix.py and
 * integrals/nuclear_attraction_integral.py. */
int gs_one_electron_grad(const double* centre, const int* l, const int* prim_off,
                         const double* expo, const double* coef, const double* comp_scale,
                         const int* func_off, const int* shell_atom, int npairs,
                         const int* pair_shells, int nbf, int natom, const double* atom_xyz,
                         const double* atom_z, const double* density,
                         const double* energy_weighted, double* grad, void* stream);

/* Spin-orbital expansion of an MO-basis two-electron tensor on the device: mo is h^4
 * doubles (chemists' order (pq|rs), row-major), out is (2h)^4 doubles, every element of
 * which is written.  mode 0 replaces spin_basis_set (matrixelements/transformations.py:
 * 73-92, spins interleaved), mode 1 blocked_spin_basis_set (29-70, alpha block first),
 * mode 2 spin_basis_anti_physicist (114-136, <rs||tu> with interleaved spins).  Results
 * are exact copies (mode 2: one subtraction) of the input elements.  Both arrays must be
 * 8-byte aligned (else GS_ERR_ARG); a 16-byte-aligned out takes the faster paired form for
 * modes 0 and 2.  h above
 * gs_spin_expand_max_orbitals() (the h x h slab one CTA stages must fit in shared memory;
 * 169 with the 227 KiB of GB300) returns GS_ERR_LIMIT; h = 0 is a no-op. */
int gs_spin_expand(const double* mo, int h, int mode, double* out, void* stream);
int gs_spin_expand_max_orbitals(void);

/* Values of every basis function at npts grid points: phi[g*nbf + f] (row-major, npts x
 * nbf), points[3*g..] in bohr; shells as in gs_pairs_build plus comp_scale[nshell*6] and
 * func_off[nshell].  Replaces Basis.value / PrimitiveBasis.value
 * (objects/basis_function.py, objects/primitive_basis_function.py:44-60) as the
 * reference's exchange-correlation quadrature calls them (kohnsham/integration.py:14-51). */
int gs_basis_on_grid(const double* centre, const int* l, const int* prim_off, const double* expo,
                     const double* coef, const double* comp_scale, const int* func_off,
                     int nshell, int nbf, long long npts, const double* points, double* phi,
                     void* stream);

/* LDA functionals at npts densities rho[g] with quadrature weights w[g]:
 *   weighted_potential[g] = w[g] * (v_x + v_c)(rho[g]),
 *   weighted_energy[g]    = w[g] * rho[g] * (eps_x + eps_c)(rho[g]),
 * Slater exchange with slater_alpha (0 = none; kohnsham/exchange/slater_exchange.py) and,
 * if vwn != 0, Vosko-Wilk-Nusair correlation with fit (a, x0, b, c), a in Rydberg as the
 * reference passes it (kohnsham/correlation/local_density.py, kohnsham/kohn_sham.py:21-28).
 * rho <= 1e-300 contributes 0 (the reference's zero-density rule, extended to subnormal
 * densities whose Wigner-Seitz radius overflows).  4c - b^2 <= 0 with vwn set is
 * GS_ERR_ARG. */
int gs_lda_xc(long long npts, const double* rho, const double* weights, double slater_alpha,
              int vwn, double vwn_a, double vwn_x0, double vwn_b, double vwn_c,
              double* weighted_potential, double* weighted_energy, void* stream);

/* Point-group zero screening of a dense n^4 tensor (row-major, device), in place: every
 * element Symmetry.none_zero_integral (common/symmetry.py:18-47) declares zero is set to
 * 0.  Tables of a non-C1 group with nops operations besides the identity:
 * table[f*nops + m] = signed 1-based image of function f under operation m+1, 0 for none
 * (the reference's basis_set_symmetry_matrix without its label row and identity column);
 * flip[m*8 + p] = 1 if operation m+1 changes parity vector p (bit 0 x, bit 1 y, bit 2 z;
 * from symmetry_exponent_dict); centre_id[f] (equal for functions on one centre);
 * parity[f] = parity bits of f's integral exponents. */
int gs_symmetry_zero(int n, int nops, const int* table, const unsigned char* flip,
                     const int* centre_id, const int* parity, double* tensor, void* stream);

/* Bytes of workspace gs_fock_jk_batched_persistent needs for ntask tasks. */
long long gs_fock_jk_persistent_workspace(int ntask);

/* Batched J/K of many molecules with every angular-momentum class in one persistent launch
 * per precision: the work distribution of TwoElectronRepulsion.create_repulsion_matrix over
 * multiprocessing.Pool.starmap (matrixelements/electron_repulsion_matrix.py:35-39) and the
 * Fock contraction of FockMatrixRestricted.create (hartreefock/fock_matrix.py:12-22).
 * tasks: the unique quartets of all molecules, grouped by canonical class; class_start is a
 * HOST array of 22 entries, the start of each canonical class's segment (class order
 * (00|00), (10|00), (10|10), (11|00) ... (22|22)) and the task count last.  One partition
 * pass drops quartets with density-weighted bound (Schwarz q_bra q_ket times the largest |P|
 * of the six shell blocks, from molecule m's table at mol_dmax + mol_sbase[m]) below
 * screen_thr (0: only exact zeros) and sends those below mixed_cut to FP32 (0: all FP64);
 * then one FP64 and one FP32 persistent kernel stride over tiles of 32 quartets (small
 * classes) or single quartets (warp form) of all classes.  Other arguments as
 * gs_fock_jk_batched_mixed. */
int gs_fock_jk_batched_persistent(const void* pair_rec, const void* prim64, const void* prim32,
                                  const double* comp_scale, const int* func_off,
                                  const int* shell_mol, const long long* mol_base,
                                  const int* mol_n, const double* mol_dmax,
                                  const int* mol_shell0, const int* mol_nshell,
                                  const long long* mol_sbase, long long mat_stride,
                                  const int* class_start, int ntask, const int* tasks,
                                  const double* pj, double* j, int nk, const double* pk,
                                  double* k, double screen_thr, double mixed_cut,
                                  void* workspace, long long ws_bytes, void* stream);

/* Dense N^4 ERI tensor from unique shell-quartet blocks: the 8-fold expansion of
 * TwoElectronRepulsion.create_repulsion_matrix (matrixelements/electron_repulsion_matrix.py:
 * 43-45).  quartets[4*q..4*q+3] = shells (A, B, C, D) of block q; its n_A n_B n_C n_D values
 * (row-major) start at vals[offsets[q]]; l and func_off per shell; out is n^4 doubles
 * (C order), every element written at least once when the quartets cover all unique ones. */
int gs_dense_expand(long long nq, const int* quartets, const long long* offsets,
                    const double* vals, const int* l, const int* func_off, int n, double* out,
                    void* stream);

/* FMA throughput probe (FP64 or FP32) used to measure the roofline peaks; sink must hold
 * blocks*threads elements of the chosen type.  No reference counterpart. */
int gs_fma_probe(int precision, int blocks, int threads, int iters, void* sink, void* stream);

/* The same probe with only the first `lanes` (1..32) lanes of each warp running the FMA
 * chains: on GB300 the FP64 time does not shrink with fewer active lanes, which is why the
 * warp kernels fill narrow recursion levels with several primitive quartets.  No
 * reference counterpart. */
int gs_fma_probe_lanes(int precision, int blocks, int threads, int iters, int lanes, void* sink,
                       void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GAUSSIUM_GB300_H */
