// mma.h -- internal interface of the GB300 MMA optimiser (mma.cu).
#pragma once
#include "le.h"

namespace topo {
struct TopoMMA;
struct GenSubGx {
    double v[8];
};
int mma_create(TopoMMA **out, int n, int m, const double *a, const double *c, const double *d);
void mma_destroy(TopoMMA *mm);
int mma_set_asymptotes(TopoMMA *mm, double init, double dec, double inc);
int mma_movelimit_dev(TopoMMA *mm, double Xmin, double Xmax, double movlim, const double *x, double *xmin,
                      double *xmax);
int mma_update_dev(TopoMMA *mm, double *xval, const double *dfdx, const double *gx, const double *dgdx,
                   const double *xmin, const double *xmax);
int mma_design_change_dev(TopoMMA *mm, const double *x, double *xold, double *ch);
int mma_kkt_dev(TopoMMA *mm, const double *x, const double *dfdx, const double *fx, const double *dgdx,
                const double *xmin, const double *xmax, double *norm2, double *normInf);
// restart constructor MMA(n, m, itr, xo1, xo2, U, L[, a, c, d]) (MMA.cc:6-178):
// the iteration counter and the histories and asymptotes of an earlier run
int mma_restart_set_dev(TopoMMA *mm, int itr, const double *xo1, const double *xo2, const double *U, const double *L);
// MMA::Restart (MMA.cc:307-350)
int mma_restart_get_dev(TopoMMA *mm, double *xo1, double *xo2, double *U, double *L);
int mma_n(const TopoMMA *mm);
int mma_m(const TopoMMA *mm);
void *mma_stream(TopoMMA *mm);
}  // namespace topo
