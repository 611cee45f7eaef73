/*
 * wtb_gpu.h -- C ABI of the GB300 exciton path (libwtb_gb300.so).
 *
 * The entry points replace the Fortran subroutines of the WTB exciton path one for one; each
 * declaration names the reference interface it stands in for (file:line inside the WTB sources).
 * Conventions shared by every call:
 *   - plain pointers and sizes only; arrays use Fortran column-major order and complex(8) is
 *     interleaved (re, im) double, i.e. C99 `double _Complex`;
 *   - the caller allocates every output array; host pointers are used only during the call;
 *   - every function returns a status code (WTB_OK = 0); wtb_last_error() returns the text the
 *     reference would have printed before its STOP;
 *   - a context binds one CUDA device and one stream; it is not thread-safe (one per host thread).
 */
#ifndef WTB_GPU_H
#define WTB_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wtb_ctx wtb_ctx;

/* status codes */
#define WTB_OK 0
#define WTB_EBADARG 1   /* invalid argument / band window outside the occupied or empty states */
#define WTB_ENOMEM 2    /* device allocation failed */
#define WTB_ENOCONV 3   /* eigensolver did not converge within maxit */
#define WTB_ETIMEOUT 4  /* a bounded device wait gave up; the kernel returned early */
#define WTB_ENAN 5      /* non-finite value in the input or the iteration */
#define WTB_ECUDA 6     /* CUDA runtime error */
#define WTB_ESTATE 7    /* call made before the state it needs (e.g. no H(R) set) */
#define WTB_ENODEV 8    /* no usable CUDA device / kernels missing for this device */

/* arithmetic of the BSE operator (the Rayleigh-Ritz, orthogonalisation and final refinement are FP64 in
 * every mode) */
#define WTB_PREC_FP64 0   /* plain FP64 form: FP64 operator, FP64 iteration */
#define WTB_PREC_FP32 1   /* FP32 operator (CUDA cores), FP32 iteration vectors */
#define WTB_PREC_BF16X3 2 /* split-BF16 tensor-core operator, 3 slice products, FP32 accumulation */
#define WTB_PREC_BF16X6 3 /* split-BF16 tensor-core operator, 6 slice products (~FP32 accuracy) */

/* how the BSE operator is applied */
#define WTB_OP_DENSE 0   /* dense Hamiltonian built in HBM, dense matvecs */
#define WTB_OP_MATFREE 1 /* V(k,k') table and band vectors only; the matvec recomputes the kernel */

/* Coulomb potentials (COULOMB_POT key; select case at src/module_bse.F90:49-72) */
#define WTB_V2DK 0
#define WTB_V3D 1
#define WTB_V3DL 2
#define WTB_V2DT 3
#define WTB_V2DT2 4
#define WTB_V2DOH 5
#define WTB_V2DRK 6
#define WTB_V1DT 7
#define WTB_V0DT 8

/* Run keys of bsesolver/bsedielraw (src/module_bse.F90:2023-2026, :835; defaults at
 * src/module_input.F90:54-122).  Matches a Fortran bind(C) derived type field by field. */
typedef struct wtb_bse_params {
  int ngrid[3];      /* NGX NGY NGZ */
  int nc, nv;        /* NBANDSC NBANDSV */
  double mshift[3];  /* SHIFT_1..3 */
  int coultype;      /* WTB_V2DRK, ... */
  int renorm;        /* RNMD (imagrenorm) */
  double ktol;       /* KTOL */
  double ediel[3];   /* EDIEL_T EDIEL EDIEL_B */
  double ez, w_coul, r0, lc; /* EDIEL_Z W_COUL R_0 LC */
  double cshift;     /* CSHIFT: optics denominator and Lorentzian width */
  double ebse0, ebsef; /* ENSPECI ENSPECF */
  int numbse;        /* NESPEC */
  int nev;           /* number of excitons (the reference hard-codes 100) */
  int precision;     /* WTB_PREC_* */
  int op;            /* WTB_OP_* */
  double tol;        /* relative residual target of the eigensolver (SLEPc uses 1e-8) */
  int maxit;         /* iteration cap (SLEPc uses 200) */
  int block;         /* eigensolver block size, 0 = automatic */
} wtb_bse_params;

/* Per-call measurements filled by the solver entry points (may be NULL). */
typedef struct wtb_timings {
  double t_bands_ms, t_build_ms, t_solve_ms, t_optics_ms, t_total_ms;
  int iterations, matvec_columns;
  double max_rel_residual;
  double refine_shift_max; /* max |E_refined - E_iteration| in eV from the FP64 final step */
  int kernel_launches;
} wtb_timings;

/* ---------------------------------------------------------------------------------------------- */
/* context */
int wtb_ctx_create(wtb_ctx** ctx, int device);
int wtb_ctx_destroy(wtb_ctx* ctx);
const char* wtb_last_error(const wtb_ctx* ctx);
int wtb_version(void);

/* Replaces the module globals filled by hamiltonian_input_read
 * (src/module_hamiltonian.F90:8-31, :35-194): w90basis, nvec, ffactor, rvec, hopmatrices,
 * ihopmatrices, rlat, efermi, scs and systype ("NP" doubles the spectrum, src/module_bse.F90:875-879).
 *   rvec        nvec x 3, integer lattice coordinates      (rvec(iR,d))
 *   hopmatrices nvec x w x w, Re H_mn(R) at (iR,m,n)        (hopmatrices(iR,m,n))
 *   rlat        3 x 3, rlat(i,:) = lattice vector a_i        (Angstrom) */
int wtb_set_hr(wtb_ctx* ctx, int w90basis, int nvec, const int* rvec, const int* ffactor,
               const double* hopmatrices, const double* ihopmatrices, const double* rlat, double efermi,
               double scs, int systype_np);

/* Replaces eigsys (src/module_hamiltonian.F90:200-320) with its full argument list: H(k) Fourier sum,
 * Hermitian eigensolve, autovetores(i,:) = i-th eigenvector, nocp = #(E <= 0), scissor scs above nocp.
 * Stateless: runs on the process-wide default context (device 0).  `exc` and `nthreads` are accepted
 * and ignored, as in the reference. */
int wtb_eigsys(int nthreads, double scs, double exc, int* nocp, const int* ffactor, double kx, double ky,
               double kz, int w90basis, int nvec, const double* rlat, const int* rvec, const double* hopmatrices,
               const double* ihopmatrices, double efermi, double* energias, double* autovetores);

/* Replaces monhkhorst_pack (src/module_kmesh.F90:338-386): kpt is n1*n2*n3 x 3. Host computation. */
int wtb_monhkhorst_pack(int n1, int n2, int n3, const double* shift, const double* rlat1, const double* rlat2,
                        const double* rlat3, double* kpt);

/* Replaces the eigsys loop of bsesolver (src/module_bse.F90:2230-2245) plus the band checks of
 * quantumnumbers2 (src/module_math.F90:362-368): eigv(nk, nv+nc), vector(nk, nv+nc, w), nocpk(nk).
 * Any output pointer may be NULL; the bands stay resident on the device for later calls. */
int wtb_eigsys_mesh(wtb_ctx* ctx, int nk, const double* kpt, int nv, int nc, double* eigv, double* vector,
                    int* nocpk);

/* Replaces the scalar potentials of module_coulomb (v2dk, vcoul, v3diel, v2dt, v2dt2, v2dohono, v2drk,
 * v0dt; src/module_coulomb.F90:11-387) evaluated for every pair: V(n1, n2) with V(i,j) = v(kpt1(i,:),
 * kpt2(j,:)). */
int wtb_coulomb_table(wtb_ctx* ctx, const wtb_bse_params* p, int n1, const double* kpt1, int n2,
                      const double* kpt2, double* V);

/* Replaces one call of a scalar potential of module_coulomb with its explicit lattice argument, e.g.
 * real(8) function v2drk(kpt1,kpt2,ngrid,rlat,ediel,lc,ez,w,r0,tolr) (src/module_coulomb.F90:286) or
 * v3diel(kpt1,kpt2,ediel,rlat,ngrid,tolr) (:98): v = V(kpt1, kpt2) for the potential p->coultype with the keys
 * of p (ngrid, ktol = tolr, ediel, ez, w_coul, r0, lc) and rlat(3, 3) (rlat(i,:) = a_i).  Evaluated by the
 * library's Coulomb kernel on the process-wide default context (device 0), like wtb_eigsys. */
int wtb_coulomb_pair(const wtb_bse_params* p, const double* rlat, const double* kpt1, const double* kpt2, double* v);

/* Replaces the optsp/hlm loop of bsesolver (src/module_bse.F90:2317-2348; src/module_optics.F90:12-167):
 * hr(dim, 5) = hrx, hry, hrz, hrsp, hrsm for the bands of the last wtb_eigsys_mesh/wtb_bsesolver call. */
int wtb_optsp(wtb_ctx* ctx, const wtb_bse_params* p, double* hr);

/* Replaces hlm(kx,ky,kz,ffactor,w90basis,nvec,rlat,rvec,hopmatrices,ihopmatrices,hx,hy,hz)
 * (src/module_optics.F90:12-108) with its argument list: hx, hy, hz (w x w complex(8), column-major) =
 * sum_R i R_a e^{ik.R} H(R)/ndegen at one k-point, phases and R_a rounded to single precision.  Stateless, on the
 * process-wide default context (device 0), like wtb_eigsys. */
int wtb_hlm(double kx, double ky, double kz, const int* ffactor, int w90basis, int nvec, const double* rlat,
            const int* rvec, const double* hopmatrices, const double* ihopmatrices, double* hx, double* hy, double* hz);

/* Replaces optsp(ev,vv,ec,vc,kx,ky,kz,ffactor,sme,w90basis,nvec,rlat,rvec,hopmatrices,ihopmatrices,hrx,hry,hrz)
 * (src/module_optics.F90:113-167) with its argument list: for the valence and conduction vectors vv, vc (w
 * complex(8)) with energies ev, ec, hr_a = <c|dH/dk_a|v> Re(1/(ec - ev + i sme)) (sme in single precision, the
 * reference's 1./esp assigned to a real), each one complex(8).  Stateless, on the default context. */
int wtb_optsp_pair(double ev, const double* vv, double ec, const double* vc, double kx, double ky, double kz,
                   const int* ffactor, double sme, int w90basis, int nvec, const double* rlat, const int* rvec,
                   const double* hopmatrices, const double* ihopmatrices, double* hrx, double* hry, double* hrz);

/* Replaces optdiel(rtype,vc,dimse,ngrid,elux,exciton,fosc,sme,rpart,ipart) (src/module_optics.F90:171-255) with
 * its argument list: the Lorentzian sums at one photon energy elux over the dimse energies exciton and strengths
 * fosc, width sme + avgsme(exciton) (:313-335); rpart = delta + C sum f (E - elux)/eaux, ipart = C sum f smef/eaux,
 * delta = 1 for rtype 1.  On the default context. */
int wtb_optdiel(int rtype, double vc, int dimse, const int* ngrid, double elux, const double* exciton,
                const double* fosc, double sme, double* rpart, double* ipart);

/* Replaces the matrizelbse build loop and Hermitian mirror (src/module_bse.F90:24-83, :2392-2415):
 * builds the dense BSE Hamiltonian on the device in p->precision (FP64 or FP32) from the bands of the
 * last wtb_eigsys_mesh call.  If hbse is not NULL the dim x dim complex(8) matrix is copied out. */
int wtb_bse_build(wtb_ctx* ctx, const wtb_bse_params* p, double* hbse);

/* Applies the BSE operator of the last band set-up without storing it (or from the dense build):
 * Y(dim, ncol) = H X(dim, ncol), complex(8), 1 <= ncol <= 32, in p->op / p->precision.  The operator is
 * the one the matrizelbse loop assembles (src/module_bse.F90:24-83, :2392-2415); this entry lets a caller
 * drive its own eigensolver, as the reference hands hbse to SLEPc (src/module_slepc_solver.F90:44-74). */
int wtb_bse_matvec(wtb_ctx* ctx, const wtb_bse_params* p, int ncol, const double* X, double* Y);

/* Replaces slepc_solver(HX, EX, HE, NX, NE) (src/module_slepc_solver.F90:12-97): the lowest NE eigenpairs
 * of the dense Hermitian NX x NX matrix HX (host, complex(8)); EX(NE), HE(NX, NE).  tol 1e-8 relative
 * residual and 200 iterations as in the reference, FP64 throughout. */
int wtb_slepc_solver(wtb_ctx* ctx, const double* HX, double* EX, double* HE, int NX, int NE);

/* Replaces dielbsev/dielbsep (src/module_bse.F90:171-245): activity(i) = |sum_j A(j,i) h(j)|^2 (pair = 0)
 * or Re[(sum_j A(j,i) h1(j)) conj(sum_j A(j,i) h2(j))] (pair = 1) for i <= dimse1, zero above. */
int wtb_dielbse(wtb_ctx* ctx, int dimse, int dimse1, const double* excitonvec, const double* hopt1,
                const double* hopt2, int pair, double* activity);

/* Replaces bsesolver (src/module_bse.F90:2023-2594) without its text files: mesh, bands, optics, BSE
 * operator, lowest p->nev excitons, oscillator strengths.  Outputs (each may be NULL):
 *   Ws(dim)      exciton energies, rows past nev set to 0 (the reference leaves them unassigned)
 *   acts(dim, 8) xx yy zz xy xz yz sp sm activities, rows past nev zero
 *   HE(dim, nev) exciton eigenvectors (complex(8)) */
int wtb_bsesolver(wtb_ctx* ctx, const wtb_bse_params* p, double* Ws, double* acts, double* HE, wtb_timings* t);

/* Replaces bsedielraw (src/module_bse.F90:835-1036 with optdiel, avgsme and imagrenorm,
 * src/module_optics.F90:171-401): dielf(numbse, 3, 6) = (omega, eps1, eps2) for xx yy zz xy xz yz from
 * the dimse rows of Ws and acts(dimse, 6). */
int wtb_bsedielraw(wtb_ctx* ctx, const wtb_bse_params* p, int dimse, const double* Ws, const double* acts,
                   double* dielf);

/* Replaces bsedielrawpol (src/module_bse.F90:1043-1199): dielf(numbse, 3, 5) = (omega, eps1, eps2) for the
 * xx yy zz sp sm (sigma+/sigma-) components from Ws and acts(dimse, 5) (the columns of bse_opt_diel-pol.dat);
 * every component takes optdiel's rtype 1 (eps1 = 1 + ...), then imagrenorm and the spin factor. */
int wtb_bsedielrawpol(wtb_ctx* ctx, const wtb_bse_params* p, int dimse, const double* Ws, const double* acts,
                      double* dielf);

/* Replaces spoptics (src/module_bse.F90:4802-5071) without its text files; bsesolver writes the same records
 * (:2317-2357).  For the Monkhorst-Pack mesh of p (ngrid, mshift, nv, nc; cshift is optsp's sme): bands and
 * velocity matrix elements on the device, then the dimsp = Nk nc nv independent-particle transitions as
 * REAL(4) records, column-major like the reference's vecres(dimsp, 15):
 *   kx ky kz, nocp, nocp-nv+c, nocp-nv+v, E_c-E_v, xx yy zz xy xz yz, sp sm
 * (xx = |h_x|^2, xy = Re(h_x h_y*), sp = |h_+|^2, ...), stably sorted by E_c-E_v as Bubblem sorts them
 * (src/module_math.F90:287-308).  Columns 7-13 are sp_optics.dat, columns 7-10 and 14-15 sp_optics-pol.dat. */
int wtb_spoptics(wtb_ctx* ctx, const wtb_bse_params* p, float* rec);

/* Replaces spoptpolbz (src/module_bse.F90:4532-4797) without its text files: for each k-point of the mesh of p
 * (column-major act(nk, 6)) the BZ-resolved optical activity summed over the nc x nv transitions,
 * |<c|dH/dk_a|v> / (E_c - E_v + i sme)|^2 for x y z (optspbz, src/module_optics.F90:257-311; sme = p->cshift),
 * the circular sp / sm activities and the dichroism (sp - sm)/(sp + sm) — the last column of bz_act_*.dat and
 * dichroism.dat.  An insulator is required (the same occupied count at every k-point). */
int wtb_spoptpolbz(wtb_ctx* ctx, const wtb_bse_params* p, double* act);

/* Replace spdielraw and spdielrawpol (src/module_bse.F90:4090-4308, :4318-4524): the broadened
 * independent-particle spectrum of the dimsp transitions esp with acts(dimsp, 6) = xx yy zz xy xz yz
 * (dielf(numbse, 3, 6), rtype 1 for xx yy zz) or acts(dimsp, 5) = xx yy zz sp sm (dielf(numbse, 3, 5),
 * rtype 1 for all); optdiel, avgsme, imagrenorm and the spin factor as in bsedielraw. */
int wtb_spdielraw(wtb_ctx* ctx, const wtb_bse_params* p, int dimsp, const double* esp, const double* acts,
                  double* dielf);
int wtb_spdielrawpol(wtb_ctx* ctx, const wtb_bse_params* p, int dimsp, const double* esp, const double* acts,
                     double* dielf);

/* Replaces kpathbse (src/module_kmesh.F90:124-193), host arithmetic: the Q path of bsebnds from nks corner
 * points ks(nks, 3) (reduced coordinates, column-major; taken in pairs (start, end) of segments) with npts
 * points per segment: qpath(nq, 4), nq = (nks/2) npts, column 1 the normalised path coordinate, columns 2-4
 * the Cartesian Q. */
int wtb_kpathbse(const double* rlat1, const double* rlat2, const double* rlat3, int nks, const double* ks, int npts,
                 double* qpath);

/* Replaces the matrizelbsekq build loop of bsebnds (src/module_bse.F90:452-569, :1400-1410) for one Q-path row
 * q4 = (path coordinate, Qx, Qy, Qz): the dense finite-Q BSE matrix over the mesh of p, conduction states on
 * the Q-shifted mesh (monhkhorst_packq), the exchange term -V(Q,0)<c_i|v_i><v_j|c_j> for |Q| != 0.
 * hbse(dim, dim) complex(8), full Hermitian (the reference fills the upper triangle).  dim <= 20000. */
int wtb_bse_build_q(wtb_ctx* ctx, const wtb_bse_params* p, const double* q4, double* hbse);

/* bsebnds with bsewf (src/module_bse.F90:1427-1438, ZHEEV 'V'): for one Q-path row q4 all dim eigenvalues W of the
 * finite-Q matrix and the eigenvectors il .. il+nvec-1 (1-based, the reference's excwf0..excwff) into Z(dim, nvec)
 * (complex(8), column-major), for excwfi2. */
int wtb_bse_q_eigenpairs(wtb_ctx* ctx, const wtb_bse_params* p, const double* q4, int il, int nvec, double* W,
                         double* Z);

/* Replaces the Q loop of bsebnds (src/module_bse.F90:1206-1566, ZHEEV 'N' at :1439-1447): for each of the nq
 * rows of qpath (as wtb_kpathbse writes it), all dim eigenvalues of the finite-Q matrix, ascending, into
 * exk(dim, nq) (the columns of bands_bse.dat).  FP64 throughout. */
int wtb_bsebnds(wtb_ctx* ctx, const wtb_bse_params* p, int nq, const double* qpath, double* exk);

/* Replaces LAPACK ZHEEV('N', 'U', n, A, lda, W, ...) of the dense full-spectrum paths: all eigenvalues of the
 * Hermitian n x n matrix whose upper triangle A (host, complex(8), column-major, leading dimension lda) holds,
 * ascending, in W(n).  Householder tridiagonalisation and bisection on the device, FP64. */
int wtb_zheev(wtb_ctx* ctx, int n, const double* A, int lda, double* W);

/* Replaces LAPACK ZHEEV('V', 'U', n, A, lda, W, ...): all eigenvalues W(n), ascending, and the orthonormal
 * eigenvectors Z(n, n) (complex(8), column-major, column k for W(k)) of the Hermitian matrix in A's upper
 * triangle.  Householder tridiagonalisation, bisection, inverse iteration (near-degenerate clusters
 * reorthogonalised) and the back-transformation on the device, FP64.  Eigenvectors carry an arbitrary phase
 * each, as LAPACK's do. */
int wtb_zheev_vectors(wtb_ctx* ctx, int n, const double* A, int lda, double* W, double* Z);

/* Temperature run keys of bsesolvertemp (src/module_bse.F90:2649-2652). */
typedef struct {
  double temp;  /* K; 0 is read as 1e-8 as fermidisteh does */
  int ta;       /* gap correction: 0 "FA" none, 1 "VE" gapcortemp, 2 "BE" gapcortemp2 (src/module_math.F90:383-403) */
  double st, phavg;  /* their parameters */
  int dtfull;   /* 1: xy xz yz activities computed, 0: written as zero */
  int cpol;     /* 1: sp sm activities computed, 0: written as zero */
} wtb_temp_params;

/* Replaces bsesolvertemp (src/module_bse.F90:2649-3263) without its text files: bands with the scissor
 * scs + tcor, the (f_v - f_c)-weighted BSE matrix of matrizelbsetemp (:575-660) as ZHEEV 'U' reads its upper
 * triangle, ALL its dim eigenpairs (ZHEEV 'V'), and dielbseptemp's activities (:784-810) of every exciton.
 * Outputs (each may be NULL): Ws(dim) ascending; acts(dim, 8) xx yy zz xy xz yz sp sm; HE(dim, dim)
 * complex(8) eigenvectors; fdeh(dim) the occupation differences.  FP64; dim <= 20000. */
int wtb_bsesolvertemp(wtb_ctx* ctx, const wtb_bse_params* p, const wtb_temp_params* tp, double* Ws, double* acts,
                      double* HE, double* fdeh);

/* Replaces the Q loop of bsebndstemp (src/module_bse.F90:1572-1990): wtb_bsebnds with the temperature keys of
 * tp — bands with the scissor scs + tcor on both meshes, the finite-Q matrix of matrizelbsekqtemp (:664-780,
 * the direct and exchange couplings weighted by f_v - f_c of the row's transition, as ZHEEV 'U' reads its upper
 * triangle) — all dim eigenvalues per Q in exk(dim, nq). */
int wtb_bsebndstemp(wtb_ctx* ctx, const wtb_bse_params* p, const wtb_temp_params* tp, int nq, const double* qpath,
                    double* exk);

/* The IPA records bsesolvertemp writes to sp_optics.dat / tm_coef.dat (src/module_bse.F90:2649-3263): as
 * wtb_spoptics, with the bands' scissor scs + tcor and the eight activity columns multiplied by f_v - f_c. */
int wtb_spoptics_temp(wtb_ctx* ctx, const wtb_bse_params* p, const wtb_temp_params* tp, float* rec);

/* ---- Output files (host writers; path = the file to create).  Records byte for byte in the reference's
 * formats: Fw.d / Ew.d / Iw.m edit descriptors as the Fortran standard defines them (the width-less I of excwf2
 * as I12), IEEE infinities as "Infinity"; the '#' header lines as list-directed records of character items
 * (a leading blank, no separators) with integers in 12-character fields.  Return WTB_EBADARG when the file
 * cannot be written. */
/* bse_opt_diel.dat (pol = 0: Ws, xx yy zz xy xz yz, 7F15.4) or bse_opt_diel-pol.dat (pol = 1: Ws, xx yy zz sp sm,
 * 6F15.4) from the Ws(dim) and acts(dim, 8) of wtb_bsesolver / wtb_bsesolvertemp (src/module_bse.F90:2132-2133,
 * :2556-2567). */
int wtb_write_bse_opt_diel(const char* path, int dim, const double* Ws, const double* acts, int pol);
/* sp_optics.dat / sp_optics-pol.dat from wtb_spoptics' rec(dimsp, 15) (src/module_bse.F90:2296-2297, :2366-2367). */
int wtb_write_sp_optics(const char* path, int dimsp, const float* rec, int pol);
/* tm_coef.dat / tm_coef-pol.dat (3F10.4,3I10.0,7F10.4 / ...,6F10.4) from the same records (:2300-2311, :2370-2377). */
int wtb_write_tm_coef(const char* path, int nk, int nc, int nv, const float* rec, int pol);
/* exc_wf_<n>.dat of excwf2 (src/module_bse.F90:374-408): nocpk(nk), kpt(nk, 3) column-major, the exciton's
 * energy and its dim = nk nc nv coefficients ewf (complex(8)).  With q4 (a Q-path row) the exc_wf_<n>_<q>.dat of
 * excwfi2 (:412-448), which adds the momentum line. */
int wtb_write_exc_wf(const char* path, int nk, int nc, int nv, const int* nocpk, const double* kpt, const double* q4,
                     int excnum, double energy, const double* ewf);
/* Replaces exclft over the rows of lifetime (src/module_bse.F90:326-370, :3271-3349): fosc(dim, 7) the columns of
 * bse_opt_diel.dat, sysdim "3D" / "2D" / "1D" with the lattice of wtb_set_hr; lft(dim, 4) radiative lifetimes (s)
 * for xx+yy+zz, xx, yy, zz.  pol = 1 replaces lifetimepol (:3353-3432): fosc(dim, 6) the columns of
 * bse_opt_diel-pol.dat, lft(dim, 6) adding sp and sm. */
int wtb_exciton_lifetime(wtb_ctx* ctx, const char* sysdim, const int* ngrid, int dim, const double* fosc, int pol,
                         double* lft);
/* exciton_lifetime.dat (1F15.4,4E15.4) from the energies and lft(dim, 4), or exciton_lifetime-pol.dat
 * (1F15.4,6E15.4) from lft(dim, 6) with pol = 1. */
int wtb_write_exciton_lifetime(const char* path, int dim, const double* energy, const double* lft, int pol);
/* List-directed files, written as gfortran's runtime writes list-directed records (a blank before the first
 * item, one blank between items except between two character items; REAL(8) as 1PG25.17E3, REAL(4) as
 * 1PG16.9E2, 4-byte integers as I11).
 * One component of bse_diel_*.dat (bsedielraw, src/module_bse.F90:926-931, :1004-1009; bsedielrawpol
 * :1130-1134, :1174-1178) or sp_diel_*.dat / sp_diel-pol_*.dat (spdielraw, spdielrawpol): the header record and
 * per photon energy the REAL(8) energy and the REAL(4) eps1, eps2 from dielf(numbse, 3) (column-major: omega,
 * eps1, eps2 — one component block of what wtb_bsedielraw / wtb_spdielraw return). */
int wtb_write_diel(const char* path, int numbse, const double* dielf);
/* bands_bse.dat of bsebnds (src/module_bse.F90:1536-1543) and bsebndstemp (:1981-1990): for each of the dim
 * bands, per Q-path point the REAL(4) path coordinate qpath(i, 1) and the REAL(8) energy exk(b, i) (column-major
 * exk(dim, nq), as wtb_bsebnds returns it), then an empty record. */
int wtb_write_bands_bse(const char* path, int nq, int dim, const double* qpath, const double* exk);
/* One of bz_act_x/y/z/sp/sm.dat or dichroism.dat of spoptpolbz (src/module_bse.F90:4754-4759): per k-point the
 * REAL(4) coordinates kpt(k, 1:3) (column-major kpt(nk, 3)) and the REAL(8) value(k) (one column of what
 * wtb_spoptpolbz returns). */
int wtb_write_bz_act(const char* path, int nk, const double* kpt, const double* value);
/* One Fortran edit descriptor applied to x (kind 'F', 'E' or 'I' with w, d (m for I)) into out (>= w+1 bytes).
 * Kind 'G' with (w, d) = (25, 17) or (16, 9): one REAL(8) or REAL(4) item of a list-directed record as above. */
int wtb_fortran_format(char kind, double x, int w, int d, char* out, int outlen);

/* Replaces bseoptprop (src/module_bse.F90:3766-3931, formulas :5075-5124): props(numbse, 6, 5) =
 * refractive index, extinction coefficient, reflectivity, absorption coefficient, energy-loss function.
 * spoptprop (:3438-3602) applies the same formulas to the spdielraw spectrum. */
int wtb_bseoptprop(wtb_ctx* ctx, int numbse, const double* dielf, double* props);

/* Replaces bseoptproppol and spoptproppol (src/module_bse.F90:3937-4084, :3608-3760): props(numbse, 5, 5)
 * for the xx yy zz sp sm spectrum dielf(numbse, 3, 5). */
int wtb_bseoptproppol(wtb_ctx* ctx, int numbse, const double* dielf, double* props);

/* Allocation-free variant of wtb_dielbse, for callers that cannot allocate device memory: their device
 * memory belongs to another allocator (a framework's caching pool, a host program's preallocated arena)
 * or they must not pay cudaMalloc's implicit device synchronisation.  It has no counterpart in the
 * reference.  Every pointer is a device pointer owned by the caller: excitonvec(dimse, dimse1) and
 * hopt1/hopt2(dimse) complex(8) in Fortran order, activity(dimse) real(8); stream may be NULL.  The
 * partial sums live in one fixed 2 MiB device array per GPU (held until the process exits), so
 * ceil(dimse/1024) * dimse1 * 4 must not exceed 262144; larger calls return WTB_EBADARG (reason on stderr).
 * All calls share that array: calls that overlap on the GPU race and must be ordered.  The first call on
 * a device looks up the array's address; make it before any stream capture.  That address belongs to the
 * device's primary context (the CUDA runtime's): call it with the primary context current, and do not reset
 * the device (cudaDeviceReset) after the first call. */
int wtb_dielbse_noalloc(int dimse, int dimse1, const double* excitonvec, const double* hopt1,
                        const double* hopt2, int pair, double* activity, void* stream);

/* Reverse-mode gradient of a loss L(E, f) through the last wtb_bsesolver call, which it requires (same
 * parameters, p->nev <= 16).  E_n are the exciton energies and f_n = |sum_j A(j,n) hrx(j)|^2 the xx
 * activities of that call (dielbsev, src/module_bse.F90:201-245).  Inputs: dL_dE(nev), dL_dfxx(nev) (either
 * may be NULL = zero).  Outputs (each may be NULL): dL_dhop, dL_dihop (nvec, w, w) in the layout of
 * hopmatrices/ihopmatrices (wtb_set_hr), and dL_dr0 (the R_0 screening length of V2DRK; 0 for the other
 * potentials).  The forward arithmetic differentiated is that of eigsys (src/module_hamiltonian.F90:200-320,
 * with the first-component-real eigenvector gauge and ZHEEV('L') reading the lower triangle), matrizelbse
 * (src/module_bse.F90:24-83), v2drk (src/module_coulomb.F90:286-350) and hlm/optsp
 * (src/module_optics.F90:12-167).  Degenerate excitons (|E_m - E_n| < 1e-9 eV) or degenerate bands have
 * no individual derivative; their mutual terms are dropped.  Not in the reference (it has no gradients).
 * t->iterations = iterations of the adjoint linear solve, t->t_total_ms = device time. */
int wtb_bse_backward(wtb_ctx* ctx, const wtb_bse_params* p, const double* dL_dE, const double* dL_dfxx,
                     double* dL_dhop, double* dL_dihop, double* dL_dr0, wtb_timings* t);

/* Least-squares spectrum loss L = sum_j (spinf eps2_xx(omega_j) - target_j)^2 on the omega grid of p
 * (ebse0..ebsef, numbse points), with eps2_xx the Lorentzian sum of bsedielraw (src/module_bse.F90:835-1036,
 * optdiel/avgsme src/module_optics.F90:171-335, no imagrenorm) over the dimse rows whose first nev hold the
 * exciton energies E and activities fxx (rows past nev are zero).  Returns L, dL/dE(nev) and dL/dfxx(nev)
 * (either may be NULL), the cotangents wtb_bse_backward takes.  1 <= nev <= 64. */
int wtb_spectrum_loss(wtb_ctx* ctx, const wtb_bse_params* p, int dimse, int nev, const double* E,
                      const double* fxx, const double* target, double* L, double* dL_dE, double* dL_dfxx);

/* ---------------------------------------------------------------------------------------------- */
/* batches of independent systems (strain variants, meshes of uneven size) */

/* One system's H(R), with the argument meanings of wtb_set_hr (hamiltonian_input_read,
 * src/module_hamiltonian.F90:35-194).  The arrays are read during wtb_batch_bsesolver only. */
typedef struct wtb_system {
  int w90basis, nvec;
  const int* rvec;             /* nvec x 3 */
  const int* ffactor;          /* nvec */
  const double* hopmatrices;   /* nvec x w x w */
  const double* ihopmatrices;  /* nvec x w x w */
  const double* rlat;          /* 3 x 3 */
  double efermi, scs;
  int systype_np;
} wtb_system;

typedef struct wtb_batch wtb_batch;

/* A batch solver on one device: one context per system plus one for the joint eigensolve.  The reference runs
 * one bsesolver per process and input; a batch of independent inputs is what its strain scans and
 * mesh-convergence series do by relaunching it.  nworkers (1..64) is kept for the ABI and not used. */
int wtb_batch_create(wtb_batch** batch, int device, int nworkers);
int wtb_batch_destroy(wtb_batch* batch);

/* wtb_bsesolver for nsys independent systems: system i uses sys[i] and p[i] (p[i].nev <= nev_stride).  With the
 * split-BF16 matrix-free forms (every p[i] the same precision, tol, maxit and block) the whole batch is one CUDA
 * graph launch: per-system set-up branches, one block eigensolve over all systems (each kernel launch covers
 * every system still iterating; converged systems are frozen), per-system oscillator strengths; the graph is
 * kept and relaunched while the batch keeps its shapes.  Other forms are solved system by system, largest
 * first.  Outputs, for the first p[i].nev excitons of system i:
 *   E[i * nev_stride + n]               exciton energies (eV)
 *   act[(i * 8 + a) * nev_stride + n]   activities a = xx yy zz xy xz yz sp sm (dielbsev/dielbsep)
 *   status[i]                           WTB_OK or the system's error (text: wtb_batch_error(batch, i))
 *   iterations[i]                       eigensolver iterations (may be NULL)
 * Returns WTB_OK when every system succeeded, else the first failing system's status.  wall_ms (may be NULL)
 * is the host wall time of the whole batch. */
int wtb_batch_bsesolver(wtb_batch* batch, int nsys, const wtb_system* sys, const wtb_bse_params* p, int nev_stride,
                        double* E, double* act, int* status, int* iterations, double* wall_ms);
const char* wtb_batch_error(const wtb_batch* batch, int i);
/* The joint split-BF16 operator of the last wtb_batch_bsesolver call (its accurate arithmetic, as in the final
 * Rayleigh-Ritz step) applied to ncol (1..16) vectors of every system: X and Y hold, system after system, the
 * dim_i x ncol complex(8) column-major blocks (wtb_bse_matvec's layout). */
int wtb_batch_matvec(wtb_batch* batch, int ncol, const double* X, double* Y);
/* Times (ms) of the last wtb_batch_bsesolver call of the joint form (t_ms has 7 entries).  Host wall:
 * t_ms[0] staging of the inputs, t_ms[1] graph capture (0 when the cached graph was reused), t_ms[2] graph run,
 * t_ms[3] read-back.  Device (events in the graph): t_ms[4] per-system set-up (bands, optics, operator data),
 * t_ms[5] joint eigensolve, t_ms[6] oscillator strengths. */
int wtb_batch_timings(const wtb_batch* batch, double* t_ms);

/* The launch shapes the autotuner chose in this process, as JSON into buf (len bytes, NUL-terminated):
 * {"build": the source hash the cache is keyed by, "cache": the cache file or null, "choices": [{"shape",
 * "param" (tile_n, gather_tile, scatter_cols), "choice", "source" (measured | cache | pinned |
 * default), "ms": [[candidate, mean ms], ...]}, ...]}.  Returns the full length.  Needs no device.
 * The cache file is WTB_TUNE_CACHE ("off": none), else $XDG_CACHE_HOME or $HOME/.cache + /wtb_gb300/autotune.json;
 * WTB_TUNE=off skips every measurement and WTB_TUNE_PIN="param=value,..." pins choices. */
int wtb_autotune_report(char* buf, int len);

/* The contraction form of the context's last BSE operator: WTB_FORM_NONE (dense operator, or none built),
 * the split-BF16 tensor-core product, the FP32 or FP64 CUDA-core product, or the FP32 FFT convolution that
 * the FP32 matrix-free operator uses on a two-dimensional Monkhorst-Pack mesh of at most 64 x 64 points. */
enum { WTB_FORM_NONE = 0, WTB_FORM_TC_BF16 = 1, WTB_FORM_SIMT_F32 = 2, WTB_FORM_SIMT_F64 = 3, WTB_FORM_FFT_F32 = 4 };
int wtb_operator_form(const wtb_ctx* ctx);

/* Number of CUDA kernels this library has launched in the process (instrumentation for benchmarks). */
long long wtb_kernel_launch_count(void);

/* The cudaStream_t the context launches on (for CUDA events recorded by a caller). */
void* wtb_ctx_stream(wtb_ctx* ctx);

/* Live timing of the operator's dominant kernel (the V x Z contraction of the matrix-free operator):
 * when enabled, CUDA events bracket each launch on the context's stream.  wtb_profile_read returns the
 * summed device time, the launch count, and the algorithmic flops and bytes of those launches. */
int wtb_profile_enable(wtb_ctx* ctx, int on);
int wtb_profile_read(wtb_ctx* ctx, double* total_ms, long long* launches, double* flops, double* bytes);

#ifdef __cplusplus
}
#endif

#endif /* WTB_GPU_H */
