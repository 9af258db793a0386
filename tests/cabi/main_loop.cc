// main_loop.cc -- main.cc's design loop (main.cc:24-154) written against the C
// ABI alone: the calls a PETSc program makes through the LinearElasticity,
// Filter/PDEFilt, MMA and SOMMG shims, with host arrays as VecGetArray hands
// them out on one rank.  Built with g++ against include/topopt_gb300.h and
// linked with libtopopt_gb300.so; a GPU test compares its objectives with the
// Python mirror's.
//
//   main_loop [-nelx 16 -nely 8 -nelz 8 -nlvls 3 -ncp 2 -tsc 5 -t1 0.05
//              -maxItr 3 -objective 3 -loadsignal 1 -mixed 1 -rtol 1e-10
//              -reduction 0 -basis 4 -omega0 0.01 -volfrac 0.12 -rmin 2]
//
// Prints one line per design iteration, "It.: %03d, True fx: %.17e, ..." as
// main.cc:133 does (with every digit), and with -reduction 1 the reduced
// matrices of the SOMMG object after the last iteration.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "topopt_gb300.h"

static void check(int rc, const char *where) {
    if (rc != TOPO_OK) {
        std::fprintf(stderr, "%s: %s: %s\n", where, topo_status_str(rc), topo_last_error());
        std::exit(1);
    }
}

struct Options {  // the PETSc options main.cc reads through TopOpt (TopOpt.cc:71-300)
    int nelx = 16, nely = 8, nelz = 8, nlvls = 3, ncp = 2, tsc = 5, maxItr = 3, objective = 3, loadsignal = 1;
    int mixed = 1, reduction = 0, basis = 4;
    double t1 = 0.05, rtol = 1e-10, omega0 = 0.01, volfrac = 0.12, rmin = 2.0;
    double Emax = 1.0, Ef = 1e-9, Rmax = 1.0, Rf = 1e-3, penalK = 3.0, penalM = 1.0, dalpha = 0.0, dbeta = 1e-3;
    double Xmin = 0.0, Xmax = 1.0, movlim = 0.2, beta = 0.1, eta = 0.15;
};

static Options parse(int argc, char **argv) {
    Options o;
    for (int i = 1; i + 1 < argc; i += 2) {
        std::string k = argv[i];
        const char *v = argv[i + 1];
        int *ip = k == "-nelx" ? &o.nelx : k == "-nely" ? &o.nely : k == "-nelz" ? &o.nelz : k == "-nlvls" ? &o.nlvls
                  : k == "-ncp" ? &o.ncp : k == "-tsc" ? &o.tsc : k == "-maxItr" ? &o.maxItr
                  : k == "-objective" ? &o.objective : k == "-loadsignal" ? &o.loadsignal : k == "-mixed" ? &o.mixed
                  : k == "-reduction" ? &o.reduction : k == "-basis" ? &o.basis : nullptr;
        double *dp = k == "-t1" ? &o.t1 : k == "-rtol" ? &o.rtol : k == "-omega0" ? &o.omega0
                     : k == "-volfrac" ? &o.volfrac : k == "-rmin" ? &o.rmin : nullptr;
        if (ip)
            *ip = std::atoi(v);
        else if (dp)
            *dp = std::atof(v);
        else {
            std::fprintf(stderr, "unknown option %s\n", k.c_str());
            std::exit(2);
        }
    }
    return o;
}

int main(int argc, char **argv) {
    const Options o = parse(argc, argv);
    const int n = o.nelx * o.nely * o.nelz;
    const double Emin = o.Ef * o.Emax, Rmin = o.Rf * o.Rmax;  // TopOpt.cc:472-474

    // STEP 2: the physics (main.cc:33): LinearElasticity(da_nodes, da_elem, nu, nlvls, ncp, tsc, t1, ti,
    // objective, sInt, mInt, t0, boundaries, loadloc, reduction, basis, dalpha, dbeta, omega0, region, V0)
    topo_le_params p;
    topo_le_default_params(&p, o.nelx, o.nely, o.nelz);
    p.nu = 0.3;
    p.nlvls = o.nlvls;
    p.ncp = o.ncp;
    p.tsc = o.tsc;
    p.t1 = o.t1;
    p.ti = 1;
    p.objective = o.objective;
    p.sInt = 1;
    p.mInt = 0;
    p.boundaries = 1;
    p.loadloc = 1;
    p.reduction = o.reduction;
    p.basis = o.basis;
    p.dalpha = o.dalpha;
    p.dbeta = o.dbeta;
    p.omega0 = o.omega0;
    p.optregion = 2;
    p.hx = p.hy = p.hz = 1.0;  // DMDASetUniformCoordinates over nel elements of unit size (TopOpt.cc:261)
    p.loadsignal = o.loadsignal;
    p.mixed = o.mixed;
    p.rtol = o.rtol;
    topo_le *physics = nullptr;
    check(topo_le_create(&physics, &p), "LinearElasticity");

    // filter (main.cc:51): filter = 2, the PDE filter of radius rmin
    topo_pdefilt *filter = nullptr;
    check(topo_pdefilt_create(&filter, o.nelx + 1, o.nely + 1, o.nelz + 1, 1.0, 1.0, 1.0, o.rmin, 1e-10, 5000),
          "PDEFilt");

    // STEP 5: MMA (main.cc:54-58)
    topo_mma *mma = nullptr;
    check(topo_mma_create(&mma, n, 1, nullptr, nullptr, nullptr), "MMA");
    check(topo_mma_set_asymptotes(mma, 0.1, 0.6, 1.05), "SetAsymptotes");

    // design vectors (TopOpt.cc:495-515): x = xTilde = xPhys = volfrac
    std::vector<double> x(n, o.volfrac), xTilde(n, o.volfrac), xPhys(n, o.volfrac), xold(n, o.volfrac);
    std::vector<double> dfdx(n), dgdx(n), xmin(n), xmax(n);

    // STEP 6: filter the initial design (main.cc:61)
    check(topo_filter_project(filter, x.data(), xTilde.data(), xPhys.data(), 0, o.beta, o.eta), "FilterProject");

    // STEP 7: the optimisation loop (main.cc:76-154)
    double ch = 1.0, fscale = 1.0;
    int itr = 0;
    while (itr < o.maxItr && ch > 0.01) {
        itr++;
        check(topo_le_complete_initial_state(physics, xPhys.data(), Emin, o.Emax, Rmin, o.Rmax, o.penalK, o.penalM),
              "CompleteInitialState");
        if (o.ncp > 1) check(topo_le_generate_checkpoints(physics), "GenerateCheckPoints");
        double fx = 0.0, gx = 0.0, mnd = 0.0;
        check(topo_le_compute_objective_sensitivities(physics, &fx, dfdx.data()), "ComputeObjectiveSensitivities");
        check(topo_le_volume_constraint(physics, &gx, dgdx.data(), xPhys.data(), o.volfrac), "VolumeConstraint");
        check(topo_filter_gradients(filter, xTilde.data(), dfdx.data(), 1, dgdx.data(), 0, o.beta, o.eta),
              "Gradients");
        check(topo_filter_mnd(filter, xPhys.data(), &mnd), "GetMND");
        if (itr == 1) fscale = 1.0 / fx;
        const double fxs = fx * fscale;
        for (double &v : dfdx) v *= fscale;  // VecScale(dfdx, fscale) on the host vector (main.cc:121)
        check(topo_mma_set_outer_movelimit(mma, o.Xmin, o.Xmax, o.movlim, x.data(), xmin.data(), xmax.data()),
              "SetOuterMovelimit");
        check(topo_mma_update(mma, x.data(), dfdx.data(), &gx, dgdx.data(), xmin.data(), xmax.data()), "Update");
        check(topo_mma_design_change(mma, x.data(), xold.data(), &ch), "DesignChange");
        std::printf("It.: %03d, True fx: %.17e, Scaled fx: %.17e, gx[0]: %.17e, ch: %.17e, mnd: %.17e\n", itr, fx,
                    fxs, gx, ch, mnd);
        if (gx > 0) ch = 1.0;  // main.cc:143-145
        check(topo_filter_project(filter, x.data(), xTilde.data(), xPhys.data(), 0, o.beta, o.eta), "FilterProject");
    }

    if (o.reduction) {  // the SOMMG object's public members after the loop (SOMMG.h:21-22)
        topo_sommg *red = nullptr;
        check(topo_sommg_create(&red, physics, o.basis), "SOMMG");
        const size_t k2 = (size_t)o.basis * o.basis;
        std::vector<double> Kr(k2), Mr(k2), Cr(k2), Pr(o.basis);
        check(topo_sommg_get(red, nullptr, Kr.data(), Mr.data(), Cr.data(), Pr.data()), "SOMMG members");
        for (int i = 0; i < o.basis; i++)
            std::printf("Kr[%d][%d]: %.17e Mr: %.17e Cr: %.17e Pr[%d]: %.17e\n", i, i, Kr[i * o.basis + i],
                        Mr[i * o.basis + i], Cr[i * o.basis + i], i, Pr[i]);
        topo_sommg_destroy(red);
    }

    topo_mma_destroy(mma);
    topo_pdefilt_destroy(filter);
    topo_le_destroy(physics);
    std::printf("# Optimization has terminated\n");
    return 0;
}
