// filter.h -- internal interface of the GB300 PDE filter / projection (filter.cu).
#pragma once
#include "le.h"

namespace topo {
struct TopoPDEFilt;
int pdefilt_create(TopoPDEFilt **out, int nx, int ny, int nz, double hx, double hy, double hz, double rmin, double rtol,
                   int maxit);
void pdefilt_destroy(TopoPDEFilt *f);
long long pdefilt_nel(const TopoPDEFilt *f);
const double *pdefilt_matrix(const TopoPDEFilt *f);
int pdefilt_apply_dev(TopoPDEFilt *f, const double *x_dev, double *xout_dev);
int filter_project_dev(TopoPDEFilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev, int projection,
                       double beta, double eta);
int filter_gradients_dev(TopoPDEFilt *f, const double *xTilde_dev, double *dfdx_dev, int m, double *dgdx_dev,
                         int projection, double beta, double eta);
int filter_mnd_dev(TopoPDEFilt *f, const double *x_dev, double *mnd);
}  // namespace topo
