/+
 + ebb.gpusolver -- ebb-solve's driver with the time loop on one GB300 (D source).
 +
 + This is the swap a D maintainer makes in app/solver.d: startComputation
 + (app/solver.d:330-428) and runIntegrator (app/solver.d:38-277) are replaced by calls
 + into the GPU library through ebb.gb300; importMesh, buildMesh, partitionMesh and
 + the solver/integrator templates are no longer needed, since the whole mesh stays
 + resident on one GPU.  The command line, the files written and the printed lines are
 + ebb-solve's:
 +
 +     ebb-solve -c config.json [-s save_prefix] [--precision fp64|split|df] [--device N]
 +
 + writes save_<k>_0.esln every saveIter iterations, final_0.esln and the big-endian
 + (t, drag, lift) triples of boundaryForces.frc; SIGINT/SIGUSR1 stop the loop and
 + still write the final solution.  A failed step (the reference's EdgeException /
 + CellException, or a boundary condition without a solution) ends the run with the
 + reference edge or cell id from ebb_last_error and exit status 1.
 +
 + Build (not done here: no D compiler exists on this build machine):
 +     ldc2 -O -I<repo>/ebbcfd_gb300/d gpusolver.d ebb/gb300.d \
 +          -L-L<repo>/ebbcfd_gb300/_build -L-lebbgb300 -L-rpath=<repo>/ebbcfd_gb300/_build
 + The same program exists compiled from C++ (ebbcfd_gb300/csrc/ebb_solve.cpp).
 +/
module ebb.gpusolver;

import core.atomic : atomicLoad, atomicStore;
import core.stdc.stdio : FILE, fclose, fopen, fwrite, printf, snprintf;
import core.sys.posix.signal : SIGINT, SIGUSR1, signal;

import std.bitmanip : nativeToBigEndian;
import std.datetime.stopwatch : AutoStart, StopWatch;
import std.file : readText;
import std.getopt : getopt;
import std.string : fromStringz, toStringz;

import ebb.gb300;

static shared bool interrupted = false;

extern(C) void handle(int sig) nothrow @nogc
{
    printf("Signal received\n");
    atomicStore(interrupted, true);
}

private string fluxName(int f) { return f == EBB_FLUX_ROE ? "roeFlux" : "rusanovFlux"; }

private string integratorName(int i)
{
    switch (i)
    {
        case EBB_INT_RK2: return "RK2";
        case EBB_INT_RK2_TVD: return "RK2_TVD";
        case EBB_INT_RK4: return "RK4";
        default: return "Euler";
    }
}

/// prints what the library reports about a failed call and returns 1
private int failed(string what, int code, ebb_solver* s)
{
    char[256] msg = 0;
    int kind;
    long index = -1;
    if (s !is null)
        ebb_last_error(s, &kind, &index, msg.ptr, msg.length);
    printf("Solver encountered an error: %s (status %d): %s", what.toStringz, code, msg.ptr);
    if (index >= 0)
        printf(" [index %lld]", index);
    printf("\n");
    return 1;
}

private void printRecord(const ref ebb_step_record r, double t, double dt)
{
    printf("lift force = %f\t drag force = %f\t t = %f\n", r.lift, r.drag, t);
    printf("rho_RMS = %.10e\tu_RMS = %.10e\tv_RMS = %.10e\tE_RMS = %.10e\tFlux_R = %.10e\t dt = %10.10f\n",
           r.resid[0], r.resid[1], r.resid[2], r.resid[3], r.rmax, dt);
}

/// startComputation + runIntegrator on the GPU; returns the process exit status
int startComputationGpu(string configText, string saveFile, int precision)
{
    ebb_config cfg;
    char[512] err = 0;
    int r = ebb_config_parse(configText.toStringz, &cfg, err.ptr, err.length);
    if (r != EBB_OK)
        return failed(err.ptr.fromStringz.idup, r, null);
    if (!checkLayout())
        return failed("the library's struct layout differs from this binding", EBB_ERR_ARG, null);

    ebb_mesh* mesh;
    r = ebb_mesh_import(cfg.mesh_file.ptr, &mesh, err.ptr, err.length);
    if (r != EBB_OK)
        return failed(err.ptr.fromStringz.idup, r, null);
    scope (exit) ebb_mesh_free(mesh);
    ebb_mesh_info info;
    ebb_mesh_get_info(mesh, &info);

    ebb_solver* s;
    r = ebb_solver_create(mesh, &cfg, precision, &s, err.ptr, err.length);
    if (r != EBB_OK)
        return failed(err.ptr.fromStringz.idup, r, null);
    scope (exit) ebb_solver_destroy(s);

    // -s prefix: restart from rank 0's file (app/solver.d:455-458, solve.d:209-220)
    if (saveFile.length)
    {
        r = ebb_load_solution(s, saveFile.toStringz);
        if (r != EBB_OK)
            return failed("Failed to load solution " ~ saveFile, r, s);
    }

    printf("Running 2D finite volume solver\n-limited: %s\n-order: %lld\n-flux: %s\n-integrator: %s\n",
           cfg.limited ? "true".ptr : "false".ptr, cfg.order, fluxName(cfg.flux).toStringz,
           integratorName(cfg.integrator).toStringz);

    ubyte[] forces;
    ebb_step_record[] rec = new ebb_step_record[4096];
    ebb_step_record last;
    bool haveLast = false;
    long iterations = 0, saveItr = 0;
    int status = 0;
    auto sw = StopWatch(AutoStart.yes);
    while (!atomicLoad(interrupted))
    {
        // run up to the next iteration that prints or saves, 4096 at most
        long chunk = rec.length;
        foreach (k; 0 .. chunk)
        {
            const it = iterations + k;
            if ((cfg.plot_iter > 0 && it % cfg.plot_iter == 0) || (cfg.save_iter > 0 && it % cfg.save_iter == 0))
            {
                chunk = k + 1;
                break;
            }
        }
        long n;
        r = ebb_run(s, chunk, rec.ptr, &n);
        foreach (k; 0 .. n)
        {
            const ref rr = rec[k];
            forces ~= nativeToBigEndian(rr.t)[];
            forces ~= nativeToBigEndian(rr.drag)[];
            forces ~= nativeToBigEndian(rr.lift)[];
            if (cfg.plot_iter > 0 && (iterations + k) % cfg.plot_iter == 0)
                printRecord(rr, rr.t, rr.dt);
            last = rr;
            haveLast = true;
        }
        if (r != EBB_OK)
        {
            status = failed("solver step failed", r, s);
            break;
        }
        if (n > 0 && cfg.save_iter > 0 && (iterations + n - 1) % cfg.save_iter == 0)
        {
            char[512] name = 0;
            snprintf(name.ptr, name.length, "save_%lld_0.esln", saveItr++);
            if (ebb_save_solution(s, name.ptr, last.t, last.dt) != EBB_OK)
                status = failed("saving a solution failed", EBB_ERR_IO, s);
        }
        iterations += n;
        if (n < chunk)
            break; // t reached tEnd
    }
    const elapsed = sw.peek.total!"usecs" / 1e6;

    FILE* frc = fopen("boundaryForces.frc", "wb");
    if (frc !is null)
    {
        fwrite(forces.ptr, 1, forces.length, frc);
        fclose(frc);
    }
    double t, dt;
    long its;
    ebb_get_time(s, &t, &dt, &its);
    if (ebb_save_solution(s, "final_0.esln", t, dt) != EBB_OK)
        status = failed("saving the final solution failed", EBB_ERR_IO, s);
    if (haveLast)
        printRecord(last, t, dt);
    printf("total solver time: %g s\n", elapsed);
    if (iterations > 0)
    {
        const perIt = elapsed / iterations;
        printf("average time per iteration: %g s\n", perIt);
        printf("average time per cell: %g us\n", perIt / (info.n_cells + info.n_ghost) * 1e6);
    }
    printf("exiting\n");
    return status;
}

int main(string[] args)
{
    string configFile, saveFile, precisionName = "fp64";
    int device = 0;
    getopt(args, "c|config", "config file to read", &configFile,
                 "s|save", "Save file to start from", &saveFile,
                 "precision", "fp64, split or df", &precisionName,
                 "device", "GPU to run on", &device);
    signal(SIGINT, &handle);
    signal(SIGUSR1, &handle);
    if (saveFile.length)
        saveFile ~= "0.esln";
    ebb_set_device(device);
    auto sw = StopWatch(AutoStart.yes);
    const precision = precisionName == "split" ? EBB_PREC_SPLIT
                    : precisionName == "df" ? EBB_PREC_DF : EBB_PREC_FP64;
    const status = startComputationGpu(readText(configFile), saveFile, precision);
    printf("total run time: %g\n", sw.peek.total!"usecs" / 1e6);
    return status;
}
