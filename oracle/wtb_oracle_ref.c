/*
 * C restatement of the reference's element-by-element BSE build and of a dense Hermitian matvec --
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline; never linked into the product).
 *
 * oracle_build_rows follows the build loop of bsesolver (src/module_bse.F90:2399-2406): for every row
 * i of the sample and every column j >= i it calls matrizelbse (src/module_bse.F90:24-83), which
 * evaluates the selected Coulomb potential for (k_i, k_j) through a switch on the potential type
 * (src/module_bse.F90:49-72; v2drk src/module_coulomb.F90:286-350, v3diel :98-131) and two length-w
 * complex dot products (prodintsq, src/module_math.F90:74-85).  Rows are distributed over OpenMP
 * threads (the reference leaves its `!$omp parallel do` inert, src/module_bse.F90:2394).
 * oracle_dense_mv is y = H x for a row block of a dense complex(8) matrix, the operation SLEPc's
 * Krylov-Schur applies to the assembled AIJ matrix (src/module_slepc_solver.F90:44-74).
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

typedef struct {
  int coultype; /* 6 = V2DRK, 2 = V3DL, 1 = V3D */
  int ngrid[3];
  double ktol, ediel[3], ez, w, r0, lc;
  double rlat[9]; /* row-major: rlat[3*i + j] = component j of a_(i+1) */
} oracle_coul;

static double vcell2D(const double* r) {
  const double x = r[1] * r[5] - r[2] * r[4], y = r[2] * r[3] - r[0] * r[5], z = r[0] * r[4] - r[1] * r[3];
  return sqrt(x * x + y * y + z * z);
}

static double vcell3D(const double* r) {
  const double x = r[1] * r[5] - r[2] * r[4], y = r[2] * r[3] - r[0] * r[5], z = r[0] * r[4] - r[1] * r[3];
  return fabs(x * r[6] + y * r[7] + z * r[8]);
}

static double potential(const oracle_coul* p, const double* k1, const double* k2) {
  const double cic = -(double)(0.0904756f * 1000.0f);
  const double dx = k1[0] - k2[0], dy = k1[1] - k2[1], dz = k1[2] - k2[2];
  const double modk = sqrt(dx * dx + dy * dy + dz * dz);
  const double ng = (double)p->ngrid[0] * p->ngrid[1] * p->ngrid[2];
  switch (p->coultype) {
    case 6: { /* V2DRK */
      const double vbz = 1. / (ng * vcell2D(p->rlat));
      const double epar = p->ediel[1], et = p->ediel[0], eb = p->ediel[2];
      const double eta = sqrt(epar / p->ez), kappa = sqrt(epar * p->ez);
      const double pb = (eb - kappa) / (eb + kappa), pt = (et - kappa) / (et + kappa);
      if (modk < p->ktol) return 0.0;
      const double aux1 = (1.0 - (pb * pt * exp(-2.0 * modk * eta * p->lc))) * kappa;
      const double aux2 = (1.0 - (pt * exp(-eta * modk * p->lc))) * (1.0 - (pb * exp(-eta * modk * p->lc)));
      const double aux3 = p->r0 * modk * exp(-modk * p->w);
      const double ew = (aux1 / aux2) + aux3;
      return (vbz * cic) * exp(-modk * p->w) * (1.0 / ew) * (1.0 / modk);
    }
    case 2:
    case 1: { /* V3DL, V3D */
      const double vbz = 1. / (ng * vcell3D(p->rlat));
      const double ed = p->coultype == 2 ? p->ediel[1] : 1.0;
      if (modk < p->ktol) return 0.0;
      return vbz * (cic / ed) * (1.0 / (modk * modk));
    }
    default:
      return 0.0;
  }
}

/* Rows [row0, row1) of the upper triangle (j >= i), written to out[(i-row0)*dim + j].
 * eigv: nk x (nv+nc) row-major, vec: nk x (nv+nc) x w complex row-major, kpt: nk x 3 row-major. */
void oracle_build_rows(int nk, int nc, int nv, int w, const double* eigv, const zc* vec, const double* kpt,
                       const oracle_coul* p, long row0, long row1, zc* out) {
  const long dim = (long)nk * nc * nv;
  const int nb = nv + nc;
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = row0; i < row1; ++i) {
    const int ki = (int)(i / (nc * nv)), ci = (int)((i / nv) % nc), vi = (int)(i % nv);
    const zc* cvi = vec + ((size_t)ki * nb + nv + ci) * w;
    const zc* vvi = vec + ((size_t)ki * nb + vi) * w;
    for (long j = i; j < dim; ++j) {
      const int kj = (int)(j / (nc * nv)), cj = (int)((j / nv) % nc), vj = (int)(j % nv);
      const double vcoul = potential(p, kpt + 3 * ki, kpt + 3 * kj);
      zc el;
      if (i == j) {
        el = (eigv[ki * nb + nv + ci] - eigv[ki * nb + vi]) + vcoul;
      } else {
        const zc* cvj = vec + ((size_t)kj * nb + nv + cj) * w;
        const zc* vvj = vec + ((size_t)kj * nb + vj) * w;
        zc vc = 0, vv = 0;
        for (int o = 0; o < w; ++o) {
          vc += conj(cvi[o]) * cvj[o];
          vv += conj(vvi[o]) * vvj[o];
        }
        el = vcoul * vc * vv;
      }
      out[(i - row0) * dim + j] = el;
    }
  }
}

/* y[r][c] = sum_j H[r][j] x[j][c] for the nrow x dim row block H (row-major), x dim x ncol row-major. */
void oracle_dense_mv(long nrow, long dim, const zc* H, const zc* x, int ncol, zc* y) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < nrow; ++r) {
    for (int c = 0; c < ncol; ++c) {
      zc acc = 0;
      for (long j = 0; j < dim; ++j) acc += H[r * dim + j] * x[j * ncol + c];
      y[r * ncol + c] = acc;
    }
  }
}

int oracle_num_threads(void) {
  int n = 1;
#pragma omp parallel
  {
#pragma omp single
    {
#ifdef _OPENMP
      n = omp_get_num_threads();
#endif
    }
  }
  return n;
}
