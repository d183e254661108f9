// md_js -- the reference's script front end over the C ABI of libfemmd:
// the global System object (37 methods), the file helpers read_file,
// write_to_file, append_to_file, make_dir and change_dir, the DEV, PBCTYPE
// and FILECONTENT tables, then the script's mdmain().  Usage: md_js script.js
//
// Reference: femmd2D/src/interface.cpp:86-756 (the bindings, their
// registration at :647-709 and the interpreter loop at :712-756).  The
// script engine is Duktape 1.5.1 (duktape.h / duk_config.h / duktape.cpp,
// third-party code the reference vendors); this repository does not carry it,
// the build compiles it from a Duktape source directory named at build time.
//
// Differences from the reference's bindings:
//   * a failed call throws a script error carrying femmd_last_error(), which
//     ends mdmain with "Error: ..." (the reference has no checks);
//   * property averaging (Properties::compute after every step, which the
//     reference always does) is switched on at start with the reference's
//     defaults (step_avg 1000, step_equi 10000); set_equilibrium_steps and
//     set_average_average_steps change them, set_reset_properties restarts
//     the sums;
//   * set_velocities(v0) draws directions from a seeded generator (a seed per
//     call) instead of rand();
//   * set_average_steps_rdf and set_range_rdf are accepted and have no
//     effect: the RDF is outside the timestep this library implements.
#include <sys/stat.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "duktape.h"
#include "femmd.h"

namespace {

femmd_ctx *g_sys = nullptr;  // the reference's global MDSystem (interface.cpp:19)
int g_avg = 1000, g_equi = 10000;
bool g_traj = false;
int g_traj_steps = 0;
uint64_t g_seed = 12345;

// A failed library call becomes a script error.
void check(duk_context *ctx, femmd_status st, const char *what) {
    if (st != FEMMD_OK) {
        const char *msg = femmd_last_error(g_sys);
        duk_error(ctx, DUK_ERR_ERROR, "%s: %s", what, msg ? msg : "error");
    }
}

// ---------------------------------------------------------- file helpers

duk_ret_t js_write(duk_context *ctx, bool append) {
    const char *name = duk_require_string(ctx, 0);
    const char *text = duk_require_string(ctx, 1);
    std::ofstream f(name, append ? std::ios::app : std::ios::trunc);
    if (!f) duk_error(ctx, DUK_ERR_ERROR, "cannot open %s", name);
    f << text;
    return 0;
}
duk_ret_t js_write_to_file(duk_context *ctx) { return js_write(ctx, false); }
duk_ret_t js_append_to_file(duk_context *ctx) { return js_write(ctx, true); }

// read_file(name, FILECONTENT.INT | FLOAT | TEXT): whitespace-separated
// numbers as an Int32Array or Float32Array, or the text with every line
// ending in '\n'.
duk_ret_t js_read_file(duk_context *ctx) {
    const char *name = duk_require_string(ctx, 0);
    const int kind = duk_require_int(ctx, 1);
    std::ifstream f(name);
    if (!f) duk_error(ctx, DUK_ERR_ERROR, "cannot open %s", name);
    if (kind == 0 || kind == 1) {
        std::vector<int32_t> vi;
        std::vector<float> vf;
        if (kind == 0) {
            int32_t x;
            while (f >> x) vi.push_back(x);
        } else {
            float x;
            while (f >> x) vf.push_back(x);
        }
        const size_t bytes = kind == 0 ? vi.size() * sizeof(int32_t) : vf.size() * sizeof(float);
        void *buf = duk_push_fixed_buffer(ctx, bytes);
        if (bytes) std::memcpy(buf, kind == 0 ? (const void *)vi.data() : (const void *)vf.data(), bytes);
        duk_push_buffer_object(ctx, -1, 0, bytes, kind == 0 ? DUK_BUFOBJ_INT32ARRAY : DUK_BUFOBJ_FLOAT32ARRAY);
        return 1;
    }
    std::string text, line;
    while (std::getline(f, line)) {
        text += line;
        text.push_back('\n');
    }
    duk_push_lstring(ctx, text.data(), text.size());
    return 1;
}

duk_ret_t js_make_dir(duk_context *ctx) {
    mkdir(duk_require_string(ctx, 0), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH);
    return 0;
}
duk_ret_t js_change_dir(duk_context *ctx) {
    if (chdir(duk_require_string(ctx, 0)) != 0) {
        // as the reference: a directory that cannot be entered is ignored
    }
    return 0;
}

// --------------------------------------------------------------- System

duk_ret_t js_init(duk_context *ctx) {
    check(ctx, femmd_init(g_sys, duk_require_number(ctx, 0), duk_require_number(ctx, 1)), "init");
    return 0;
}
duk_ret_t js_reset(duk_context *ctx) {
    check(ctx, femmd_reset(g_sys), "reset");
    check(ctx, femmd_set_property_averaging(g_sys, 1, g_avg, g_equi), "reset");
    return 0;
}
duk_ret_t js_add_particle(duk_context *ctx) {
    check(ctx,
          femmd_add_particle(g_sys, duk_require_number(ctx, 0), duk_require_number(ctx, 1),
                             duk_require_number(ctx, 2), duk_require_number(ctx, 3), duk_require_number(ctx, 4),
                             duk_require_number(ctx, 5), duk_require_int(ctx, 6)),
          "add_particle");
    return 0;
}
// add_elastomer(vertices Float32Array (x, y pairs), triangles Int32Array
// (1-based triples), x, y, type, group, sigma, mass, exclude)
duk_ret_t js_add_elastomer(duk_context *ctx) {
    duk_size_t vb = 0, tb = 0;
    const float *v = static_cast<const float *>(duk_require_buffer_data(ctx, 0, &vb));
    const int *t = static_cast<const int *>(duk_require_buffer_data(ctx, 1, &tb));
    check(ctx,
          femmd_add_elastomer(g_sys, v, (int)(vb / (2 * sizeof(float))), t, (int)(tb / (3 * sizeof(int))),
                              duk_require_number(ctx, 2), duk_require_number(ctx, 3), duk_require_int(ctx, 4),
                              duk_require_int(ctx, 5), duk_require_number(ctx, 6), duk_require_number(ctx, 7),
                              duk_require_boolean(ctx, 8) ? 1 : 0),
          "add_elastomer");
    return 0;
}
duk_ret_t js_allocate_cuda(duk_context *ctx) {
    check(ctx, femmd_allocate_cuda(g_sys), "allocate_cuda");
    return 0;
}
duk_ret_t js_init_neighbor_list(duk_context *ctx) {
    check(ctx, femmd_init_neighbor_list(g_sys), "init_neighbor_list");
    return 0;
}
// set_pair_potential(eps, rc, ushift): Float64Arrays of numTypes^2 values
duk_ret_t js_set_pair_potential(duk_context *ctx) {
    duk_size_t be = 0, br = 0, bu = 0;
    const double *eps = static_cast<const double *>(duk_require_buffer_data(ctx, 0, &be));
    const double *rc = static_cast<const double *>(duk_require_buffer_data(ctx, 1, &br));
    const double *us = static_cast<const double *>(duk_require_buffer_data(ctx, 2, &bu));
    if (br != be || bu != be) duk_error(ctx, DUK_ERR_RANGE_ERROR, "set_pair_potential: arrays of unequal length");
    check(ctx, femmd_set_pair_potential(g_sys, eps, rc, us, (int)(be / sizeof(double))), "set_pair_potential");
    return 0;
}
duk_ret_t js_save(duk_context *ctx, int format, bool flagged, const char *what) {
    const char *name = duk_require_string(ctx, 0);
    const int append = flagged ? duk_require_int(ctx, 1) : 0;
    check(ctx, femmd_save_frame(g_sys, name, format, append), what);
    return 0;
}
duk_ret_t js_save_vtk(duk_context *ctx) { return js_save(ctx, 2, false, "save_vtk"); }
duk_ret_t js_save_vtf(duk_context *ctx) { return js_save(ctx, 3, true, "save_vtf"); }
duk_ret_t js_save_cluster_vtf(duk_context *ctx) { return js_save(ctx, 4, true, "save_cluster_vtf"); }
duk_ret_t js_save_cluster_xyz(duk_context *ctx) { return js_save(ctx, 0, true, "save_cluster_xyz"); }
// the writers form the clusters' centres of mass from the current state
duk_ret_t js_calc_cluster_props(duk_context *) { return 0; }
// the reference's doStep writes traj.xyz every trajectorySteps steps while on
void apply_trajectory(duk_context *ctx) {
    const bool on = g_traj && g_traj_steps > 0;
    check(ctx, femmd_set_trajectory(g_sys, on ? "traj.xyz" : nullptr, on ? g_traj_steps : 0, 0), "save_trajectory");
}
duk_ret_t js_save_trajectory(duk_context *ctx) {
    g_traj = duk_require_boolean(ctx, 0) != 0;
    apply_trajectory(ctx);
    return 0;
}
duk_ret_t js_set_trajectory_steps(duk_context *ctx) {
    g_traj_steps = duk_require_int(ctx, 0);
    apply_trajectory(ctx);
    return 0;
}
duk_ret_t js_run(duk_context *ctx) {
    check(ctx, femmd_run(g_sys, duk_require_int(ctx, 0)), "run");
    return 0;
}

// property order of femmd_get_properties
enum { P_UKIN, P_UPOT, P_UTOT, P_TEMP, P_VIR, P_FEAVIR, P_PRESS, P_CLUKIN, P_CLVIR, P_MOLPRESS, P_COUNT };

duk_ret_t js_print_props(duk_context *ctx) {
    double avg[P_COUNT] = {0};
    check(ctx, femmd_get_average_properties(g_sys, avg, nullptr, nullptr, nullptr, nullptr, nullptr), "print_props");
    std::printf("%d %f %f %f %f %f %f\n%f %f %f\n", femmd_get_steps(g_sys), avg[P_UKIN], avg[P_UPOT], avg[P_UTOT], avg[P_VIR],
                avg[P_FEAVIR], avg[P_PRESS], avg[P_CLUKIN], avg[P_CLVIR], avg[P_MOLPRESS]);
    return 0;
}

// get_props(): { steps, and per property { avgval, curr, stdv } }
duk_ret_t js_get_props(duk_context *ctx) {
    double avg[P_COUNT] = {0}, sd[P_COUNT] = {0}, val[P_COUNT] = {0};
    check(ctx, femmd_get_average_properties(g_sys, avg, sd, val, nullptr, nullptr, nullptr), "get_props");
    const duk_idx_t o = duk_push_object(ctx);
    duk_push_number(ctx, (double)femmd_get_steps(g_sys));
    duk_put_prop_string(ctx, o, "steps");
    struct Item {
        const char *name;
        int k;  // -1: a property the reference never sets (reads 0)
    } items[] = {{"uKinetic", P_UKIN}, {"uPotential", P_UPOT}, {"uFea", -1},        {"uBonded", -1},
                 {"uTotal", P_UTOT},   {"pressure", P_PRESS}, {"virial", P_VIR}, {"feaVirial", P_FEAVIR}};
    for (const Item &it : items) {
        const duk_idx_t b = duk_push_object(ctx);
        duk_push_number(ctx, it.k < 0 ? 0.0 : avg[it.k]);
        duk_put_prop_string(ctx, b, "avgval");
        duk_push_number(ctx, it.k < 0 ? 0.0 : val[it.k]);
        duk_put_prop_string(ctx, b, "curr");
        duk_push_number(ctx, it.k < 0 ? 0.0 : sd[it.k]);
        duk_put_prop_string(ctx, b, "stdv");
        duk_put_prop_string(ctx, o, it.name);
    }
    return 1;
}

// info(): { N, nelastomers, nbonds, ntrigs, dt, kBonds, kArea, E, box {x, y} }
duk_ret_t js_info(duk_context *ctx) {
    double v[9] = {0};
    double ly = 0.0;
    check(ctx, femmd_info(g_sys, v), "info");
    check(ctx, femmd_get_box(g_sys, &v[8], &ly), "info");
    const char *names[8] = {"N", "nelastomers", "nbonds", "ntrigs", "dt", "kBonds", "kArea", "E"};
    const duk_idx_t o = duk_push_object(ctx);
    for (int k = 0; k < 8; k++) {
        duk_push_number(ctx, v[k]);
        duk_put_prop_string(ctx, o, names[k]);
    }
    const duk_idx_t b = duk_push_object(ctx);
    duk_push_number(ctx, v[8]);
    duk_put_prop_string(ctx, b, "x");
    duk_push_number(ctx, ly);
    duk_put_prop_string(ctx, b, "y");
    duk_put_prop_string(ctx, o, "box");
    return 1;
}
duk_ret_t js_set_velocities(duk_context *ctx) {
    check(ctx, femmd_set_velocities(g_sys, duk_require_number(ctx, 0), g_seed++), "set_velocities");
    return 0;
}
duk_ret_t js_set_dt(duk_context *ctx) {
    check(ctx, femmd_set_dt(g_sys, duk_require_number(ctx, 0)), "set_dt");
    return 0;
}
duk_ret_t js_set_scale(duk_context *ctx) {
    check(ctx, femmd_set_scale(g_sys, duk_require_number(ctx, 0)), "set_scale");
    return 0;
}
duk_ret_t js_set_equilibrium_steps(duk_context *ctx) {
    g_equi = (int)duk_require_number(ctx, 0);
    check(ctx, femmd_set_property_averaging(g_sys, 1, g_avg, g_equi), "set_equilibrium_steps");
    return 0;
}
duk_ret_t js_set_average_average_steps(duk_context *ctx) {
    g_avg = (int)duk_require_number(ctx, 0);
    check(ctx, femmd_set_property_averaging(g_sys, 1, g_avg, g_equi), "set_average_average_steps");
    return 0;
}
duk_ret_t js_rdf_setting(duk_context *ctx) {
    duk_require_number(ctx, 0);
    return 0;
}
duk_ret_t js_set_reset_properties(duk_context *ctx) {
    check(ctx, femmd_set_property_averaging(g_sys, 0, g_avg, g_equi), "set_reset_properties");
    check(ctx, femmd_set_property_averaging(g_sys, 1, g_avg, g_equi), "set_reset_properties");
    return 0;
}
duk_ret_t js_get_dt(duk_context *ctx) {
    double dt = 0.0;
    check(ctx, femmd_get_dt(g_sys, &dt), "get_dt");
    duk_push_number(ctx, dt);
    return 1;
}
duk_ret_t js_set_box(duk_context *ctx) {
    check(ctx, femmd_set_box(g_sys, duk_require_number(ctx, 0), duk_require_number(ctx, 1)), "set_box");
    return 0;
}
duk_ret_t js_get_box(duk_context *ctx) {
    double lx = 0.0, ly = 0.0;
    check(ctx, femmd_get_box(g_sys, &lx, &ly), "get_box");
    const duk_idx_t o = duk_push_object(ctx);
    duk_push_number(ctx, lx);
    duk_put_prop_string(ctx, o, "x");
    duk_push_number(ctx, ly);
    duk_put_prop_string(ctx, o, "y");
    return 1;
}
// useNN(x) sets dt in the reference (interface.cpp:429-434)
duk_ret_t js_use_nn(duk_context *ctx) { return js_set_dt(ctx); }
duk_ret_t js_set_num_types(duk_context *ctx) {
    check(ctx, femmd_set_num_types(g_sys, (int)duk_require_number(ctx, 0)), "set_numTypes");
    return 0;
}
duk_ret_t js_set_gravity(duk_context *ctx) {
    check(ctx, femmd_set_gravity(g_sys, duk_require_number(ctx, 0)), "set_gravity");
    return 0;
}
duk_ret_t js_set_kbond(duk_context *ctx) {
    check(ctx, femmd_set_kbond(g_sys, duk_require_number(ctx, 0)), "set_kBond");
    return 0;
}
duk_ret_t js_set_karea(duk_context *ctx) {
    check(ctx, femmd_set_karea(g_sys, duk_require_number(ctx, 0)), "set_kArea");
    return 0;
}
duk_ret_t js_set_youngs_modulus(duk_context *ctx) {
    check(ctx, femmd_set_youngs_modulus(g_sys, duk_require_number(ctx, 0)), "set_youngs_modulus");
    return 0;
}
duk_ret_t js_dev(duk_context *ctx) {
    check(ctx, femmd_set_dev(g_sys, (int)duk_require_number(ctx, 0)), "DEV");
    return 0;
}
duk_ret_t js_pbc(duk_context *ctx) {
    check(ctx, femmd_set_pbc(g_sys, (int)duk_require_number(ctx, 0)), "PBC");
    return 0;
}

// the System methods and their argument counts (interface.cpp:656-696)
const duk_function_list_entry kSystem[] = {
    {"init", js_init, 2},
    {"reset", js_reset, 0},
    {"add_particle", js_add_particle, 7},
    {"add_elastomer", js_add_elastomer, 9},
    {"allocate_cuda", js_allocate_cuda, 0},
    {"init_neighbor_list", js_init_neighbor_list, 0},
    {"set_pair_potential", js_set_pair_potential, 3},
    {"save_vtk", js_save_vtk, 1},
    {"save_vtf", js_save_vtf, 2},
    {"calc_cluster_props", js_calc_cluster_props, 0},
    {"save_cluster_vtf", js_save_cluster_vtf, 2},
    {"save_cluster_xyz", js_save_cluster_xyz, 2},
    {"save_trajectory", js_save_trajectory, 1},
    {"set_trajectory_steps", js_set_trajectory_steps, 1},
    {"run", js_run, 1},
    {"print_props", js_print_props, 0},
    {"get_props", js_get_props, 0},
    {"info", js_info, 0},
    {"set_velocities", js_set_velocities, 1},
    {"set_dt", js_set_dt, 1},
    {"set_scale", js_set_scale, 1},
    {"set_equilibrium_steps", js_set_equilibrium_steps, 1},
    {"set_average_steps_rdf", js_rdf_setting, 1},
    {"set_average_average_steps", js_set_average_average_steps, 1},
    {"set_range_rdf", js_rdf_setting, 1},
    {"set_reset_properties", js_set_reset_properties, 1},
    {"get_dt", js_get_dt, 0},
    {"set_box", js_set_box, 2},
    {"get_box", js_get_box, 0},
    {"useNN", js_use_nn, 1},
    {"set_numTypes", js_set_num_types, 1},
    {"set_gravity", js_set_gravity, 1},
    {"set_kBond", js_set_kbond, 1},
    {"set_kArea", js_set_karea, 1},
    {"set_youngs_modulus", js_set_youngs_modulus, 1},
    {"DEV", js_dev, 1},
    {"PBC", js_pbc, 1},
    {nullptr, nullptr, 0}};

void global_function(duk_context *ctx, duk_c_function f, const char *name, duk_idx_t nargs) {
    duk_push_global_object(ctx);
    duk_push_c_function(ctx, f, nargs);
    duk_put_prop_string(ctx, -2, name);
    duk_pop(ctx);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "Usage: md_js <script.js>\n");
        return 1;
    }
    if (femmd_create(0, &g_sys) != FEMMD_OK) {
        std::fprintf(stderr, "md_js: %s\n", femmd_last_error(g_sys));
        return 1;
    }
    duk_context *ctx = duk_create_heap_default();
    if (!ctx) {
        std::fprintf(stderr, "md_js: no script heap\n");
        femmd_destroy(g_sys);
        return 1;
    }
    int rc = 0;
    femmd_set_property_averaging(g_sys, 1, g_avg, g_equi);
    duk_eval_string_noresult(ctx, "var DEV = {CPU: 0, GPU: 1};");
    duk_eval_string_noresult(ctx, "var PBCTYPE = {NOPBC: 0, XPBC: 1, XYPBC: 2};");
    duk_eval_string_noresult(ctx, "var FILECONTENT = {INT: 0, FLOAT: 1, TEXT: 2};");
    global_function(ctx, js_write_to_file, "write_to_file", 2);
    global_function(ctx, js_append_to_file, "append_to_file", 2);
    global_function(ctx, js_read_file, "read_file", 2);
    global_function(ctx, js_make_dir, "make_dir", 1);
    global_function(ctx, js_change_dir, "change_dir", 1);
    duk_push_global_object(ctx);
    duk_push_object(ctx);
    duk_put_function_list(ctx, -1, kSystem);
    duk_put_prop_string(ctx, -2, "System");
    // the script, then its mdmain()
    if (duk_peval_file(ctx, argv[1]) != 0) {
        std::printf("Error: %s\n", duk_safe_to_string(ctx, -1));
        rc = 2;
    } else {
        duk_pop(ctx);
        duk_get_prop_string(ctx, -1, "mdmain");
        if (duk_pcall(ctx, 0) != 0) {
            std::printf("Error: %s\n", duk_safe_to_string(ctx, -1));
            rc = 2;
        }
    }
    duk_pop(ctx);
    duk_destroy_heap(ctx);
    femmd_destroy(g_sys);
    return rc;
}
