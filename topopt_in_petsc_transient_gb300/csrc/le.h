// le.h -- internal interface of the GB300 LinearElasticity object (le.cu).
#pragma once
#include <string>

#include "../../include/topopt_gb300.h"

namespace topo {

typedef topo_le_params LEParams;
typedef topo_le_stats LEStats;

struct TopoLE;

void set_error(const std::string &s);
const char *last_error();

int le_create(TopoLE **out, const LEParams *p);
int le_alloc(TopoLE *le);
void le_destroy(TopoLE *le);
int le_complete_initial_state(TopoLE *le, const double *xPhys_dev, double Emin, double Emax, double Rmin, double Rmax,
                              double penalK, double penalM);
int le_generate_checkpoints(TopoLE *le);
int le_compute_objective_sensitivities(TopoLE *le, double *fx, double *dfdx_dev);
int le_get_state(TopoLE *le, int which, int j, double *host_out);
int le_get_checkpoint(TopoLE *le, int c, double *U, double *DU, double *DDU);
int le_set_output(TopoLE *le, topo_mpiio *io);
int le_set_initial_displacement(TopoLE *le, const double *U0, int on_device);
int le_get_restart_state(TopoLE *le, double *DDU0, double *LT, double *DDL0);
int le_apply_km(TopoLE *le, const double *x_dev, double *Kx_dev, double *Mx_dev);
int le_stats(TopoLE *le, LEStats *out);
long long le_nel(const TopoLE *le);
long long le_ndof(const TopoLE *le);
void *le_stream(TopoLE *le);
int le_time_apply(TopoLE *le, int precision, int warmup, int reps, double *ms);
int le_kernel_timing(TopoLE *le, int kclass, int enable, double *ms_total, long long *launches);
int le_reduced_system(TopoLE *le, double *Q, double *Kr, double *Mr, double *Pr);
int le_sommg_construct_basis(TopoLE *le, double om);
int le_gram_tc_dev(const float *Q, long long ldq, const double *W, long long ldw, long long n, int kb, double *out);
int le_basis(const TopoLE *le);
void le_damping(const TopoLE *le, double *alpha, double *beta);
void box_element_matrices(double hx, double hy, double hz, double nu, double *KE, double *ME);

}  // namespace topo
