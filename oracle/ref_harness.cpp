// ref_harness.cpp -- TEST INFRASTRUCTURE.  A command-file driver for the
// reference's own C++ classes (valeraml/femmd_old, femmd2D/src), compiled from
// the reference sources by oracle/Makefile into oracle/_ref/ref_harness.  It
// replays a scene (the same setup calls a reference script makes through
// System.*, src/interface.cpp:229-563) on MDSystem in CPU mode and dumps
// setup arrays, cell/neighbour sets, forces and trajectories, and has the
// reference's file writers (md3dsystem.cpp:232-522) write frames beside the
// output file; tests/golden/make_golden.py stores both as golden fixtures.  It stands in for the
// reference's Duktape front end (src/interface.cpp:712-756) so that skin and
// capacities can be set from C++, which the script surface cannot do.
//
// Usage: ref_harness <commands.bin> <output.bin>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <string>
#include "md3dsystem.h"

enum Op {
    OP_END = 0, OP_INIT = 1, OP_PBC = 2, OP_DT = 3, OP_NUMTYPES = 4, OP_PAIR = 5, OP_KBOND = 6,
    OP_YOUNG = 7, OP_NU = 8, OP_SKIN = 9, OP_ELASTOMER = 10, OP_PARTICLE = 11, OP_BOND = 12,
    OP_INITNN = 13, OP_CAPACITY = 14, OP_RUN = 15, OP_STEP = 16, OP_BUILDNN = 17, OP_FORCES = 18,
    OP_ELASTOMER_BONDS = 19, OP_DUMP_STATE = 20, OP_DUMP_NN = 21, OP_DUMP_SETUP = 22, OP_SETVEL = 23,
    OP_GRAVITY = 24, OP_KAREA = 25, OP_SAVE = 26, OP_SCALE = 27, OP_FEA_CPU1 = 28
};

// Bond set of an elastomer: 0 keeps the reference's bonds on every triangle
// edge (interior edges twice, src/particles.cpp:335-337); 1 keeps one bond per
// boundary edge (an edge of exactly one triangle), created in triangle order
// through the reference's public Bonds::createBond; 2 keeps none.
static int g_bond_mode = 0;

static void apply_bond_mode(MDSystem &s, int nb_before, const std::vector<int32_t> &t, int nt, int offset) {
    if (g_bond_mode == 0) return;
    Bonds &b = s.particles.bonds;
    b.bondList.resize(2 * (size_t)nb_before);
    b.bondLength.resize(nb_before);
    b.numBonds = nb_before;
    b.bondListLen = 2 * nb_before;
    if (g_bond_mode != 1) return;
    std::vector<long long> keys(3 * (size_t)nt);
    for (int i = 0; i < nt; i++) {
        int e[3][2] = {{t[3 * i], t[3 * i + 1]}, {t[3 * i], t[3 * i + 2]}, {t[3 * i + 1], t[3 * i + 2]}};
        for (int k = 0; k < 3; k++) {
            long long a = std::min(e[k][0], e[k][1]), c = std::max(e[k][0], e[k][1]);
            keys[3 * i + k] = a * 4294967296LL + c;
        }
    }
    for (int i = 0; i < nt; i++) {
        int e[3][2] = {{t[3 * i], t[3 * i + 1]}, {t[3 * i], t[3 * i + 2]}, {t[3 * i + 1], t[3 * i + 2]}};
        for (int k = 0; k < 3; k++) {
            int cnt = 0;
            for (int m = 0; m < 3 * nt; m++) cnt += keys[m] == keys[3 * i + k];
            if (cnt == 1) b.createBond(e[k][0] + offset - 1, e[k][1] + offset - 1);
        }
    }
}

static FILE *fin, *fout;

template <typename T> static T rd() {
    T v;
    if (fread(&v, sizeof(T), 1, fin) != 1) { fprintf(stderr, "ref_harness: truncated input\n"); exit(3); }
    return v;
}
template <typename T> static void rdv(std::vector<T> &v, size_t n) {
    v.resize(n);
    if (n && fread(v.data(), sizeof(T), n, fin) != n) { fprintf(stderr, "ref_harness: truncated input\n"); exit(3); }
}
template <typename T> static void wr(T v) { fwrite(&v, sizeof(T), 1, fout); }
template <typename T> static void wrv(const T *p, size_t n) { if (n) fwrite(p, sizeof(T), n, fout); }

static void dump_state(MDSystem &s) {
    wr<int32_t>(OP_DUMP_STATE);
    int N = s.N;
    wr<int32_t>(N);
    wrv((const float *)s.particles.pos.data(), 2 * (size_t)N);
    wrv((const float *)s.particles.vel.data(), 2 * (size_t)N);
    wrv((const float *)s.particles.acc.data(), 2 * (size_t)N);
    wrv((const float *)s.particles.force.data(), 2 * (size_t)N);
    float sc[6] = {s.potEnergy, s.virial, s.feaVirial, s.kinEneSum, s.vvMax, s.neighborlist.dispHi};
    wrv(sc, 6);
    wr<int32_t>(s.steps);
    wr<int32_t>(s.neighborlist.totalUpdates);
}

static void dump_nn(MDSystem &s) {
    NeighborList &nl = s.neighborlist;
    wr<int32_t>(OP_DUMP_NN);
    wr<int32_t>(nl.numCells2D.x);
    wr<int32_t>(nl.numCells2D.y);
    int nc = nl.numCells, N = s.N;
    // cells as CSR, in the reference's in-cell order
    std::vector<int32_t> start(nc + 1, 0), ids;
    for (int c = 0; c < nc; c++) {
        start[c + 1] = start[c] + nl.cellCount[c];
        for (int k = 0; k < nl.cellCount[c]; k++) ids.push_back(nl.cellContent[c * nl.maxParticlesPerCell + k]);
    }
    wrv(start.data(), nc + 1);
    wrv(ids.data(), ids.size());
    std::vector<int32_t> nstart(N + 1, 0), list;
    for (int i = 0; i < N; i++) {
        nstart[i + 1] = nstart[i] + nl.neighborCount[i];
        for (int k = 0; k < nl.neighborCount[i]; k++) list.push_back(nl.neighborList[i * nl.maxNeighborsPerParticle + k]);
    }
    wrv(nstart.data(), N + 1);
    wrv(list.data(), list.size());
}

static void dump_setup(MDSystem &s) {
    Particles &p = s.particles;
    wr<int32_t>(OP_DUMP_SETUP);
    int N = s.N;
    wr<int32_t>(N);
    wrv(p.mass.data(), N);
    wrv(p.exclusionGroupIdOfPart.data(), N);
    int nb = p.bonds.numBonds;
    wr<int32_t>(nb);
    wrv(p.bonds.bondList.data(), 2 * (size_t)nb);
    wrv(p.bonds.bondLength.data(), nb);
    int nt = (int)p.feaElements.tetras.size();
    wr<int32_t>(nt);
    for (int t = 0; t < nt; t++) wrv(p.feaElements.tetras[t].ind, 3);
    for (int t = 0; t < nt; t++) wrv(&p.feaElements.xm[t].m[0][0], 9);
    wrv(p.feaElements.refVol.data(), nt);
    int nref = (int)p.feaElements.refPos.size();
    wr<int32_t>(nref);
    wrv((const float *)p.feaElements.refPos.data(), 2 * (size_t)nref);
}

int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: ref_harness <commands.bin> <output.bin>\n"); return 2; }
    fin = fopen(argv[1], "rb");
    fout = fopen(argv[2], "wb");
    if (!fin || !fout) { fprintf(stderr, "ref_harness: cannot open files\n"); return 2; }
    MDSystem *sp = new MDSystem(0);
    MDSystem &s = *sp;
    s.DEV = CPU;
    s.scale = 1;  // MDSystem leaves scale unset until set_scale
    // frames (OP_SAVE) are written beside the output file
    std::string dir = argv[2];
    dir = dir.find('/') == std::string::npos ? std::string(".") : dir.substr(0, dir.rfind('/'));
    for (;;) {
        int32_t op = rd<int32_t>();
        if (op == OP_END) break;
        switch (op) {
        case OP_INIT: { double lx = rd<double>(), ly = rd<double>(); s.init(lx, ly); break; }
        case OP_PBC: { int p = rd<int32_t>(); s.pbcType = p == 0 ? NOPBC : p == 1 ? XPBC : XYPBC; break; }
        case OP_DT: s.dt = rd<double>(); break;
        case OP_NUMTYPES: s.particles.numTypes = rd<int32_t>(); break;
        case OP_PAIR: {
            int n2 = rd<int32_t>();
            std::vector<double> e, r, u;
            rdv(e, n2); rdv(r, n2); rdv(u, n2);
            std::vector<real> ef(e.begin(), e.end()), rf(r.begin(), r.end()), uf(u.begin(), u.end());
            s.interactions.setPairForce(ef.data(), rf.data(), uf.data());
            break;
        }
        case OP_KBOND: {
            real k = rd<double>();
            if (k > 0) { s.interactions.kBond = k; s.interactions.bondForces = true; } else s.interactions.bondForces = false;
            break;
        }
        case OP_YOUNG: {
            real E = rd<double>();
            if (E > 0) { s.interactions.E = E; s.interactions.feaForces = true; } else s.interactions.feaForces = false;
            s.interactions.setElasticConstants();
            break;
        }
        case OP_NU: s.interactions.nu = rd<double>(); s.interactions.setElasticConstants(); break;
        case OP_SKIN: s.neighborlist.setSkin(rd<double>()); break;
        case OP_ELASTOMER: {
            int nv = rd<int32_t>(), nt = rd<int32_t>();
            std::vector<float> v; std::vector<int32_t> t;
            rdv(v, 2 * (size_t)nv); rdv(t, 3 * (size_t)nt);
            real x = rd<double>(), y = rd<double>();
            int typ = rd<int32_t>(), g = rd<int32_t>();
            real sig = rd<double>(), mass = rd<double>();
            int exc = rd<int32_t>();
            int nb_before = s.particles.bonds.numBonds, offset = s.N;
            s.particles.addElastomer(v.data(), nv, t.data(), nt, x, y, typ, g, sig, mass, exc != 0);
            apply_bond_mode(s, nb_before, t, nt, offset);
            break;
        }
        case OP_ELASTOMER_BONDS: g_bond_mode = rd<int32_t>(); break;
        case OP_SETVEL: {
            std::vector<float> v;
            rdv(v, 2 * (size_t)s.N);
            for (int i = 0; i < s.N; i++) { s.particles.vel[i].x = v[2 * i]; s.particles.vel[i].y = v[2 * i + 1]; }
            break;
        }
        case OP_GRAVITY: {  // DukSystemSetGravity (interface.cpp:443-453)
            real g = rd<double>();
            if (g > 0) {
                s.interactions.gravity = g;
                s.interactions.gravityForce = true;
            } else
                s.interactions.gravityForce = false;
            break;
        }
        case OP_KAREA: {  // DukSystemSetKArea (interface.cpp:466-476)
            real k = rd<double>();
            if (k > 0) {
                s.interactions.kArea = k;
                s.interactions.areaForces = true;
            } else
                s.interactions.areaForces = false;
            break;
        }
        case OP_PARTICLE: {
            real x = rd<double>(), y = rd<double>(), vx = rd<double>(), vy = rd<double>();
            real m = rd<double>(), sig = rd<double>();
            int typ = rd<int32_t>();
            s.particles.addParticle(x, y, vx, vy, m, sig, typ);
            break;
        }
        case OP_BOND: { int i = rd<int32_t>(), j = rd<int32_t>(); s.particles.bonds.createBond(i, j); break; }
        case OP_INITNN: s.neighborlist.init(); break;
        case OP_CAPACITY: {
            int ppc = rd<int32_t>(), nbr = rd<int32_t>();
            s.neighborlist.maxParticlesPerCell = ppc;
            s.neighborlist.maxNeighborsPerParticle = nbr;
            s.neighborlist.allocate();
            break;
        }
        case OP_RUN: s.integrator.run(rd<int32_t>()); break;
        case OP_STEP: s.integrator.doStep(); break;
        case OP_BUILDNN: s.neighborlist.buildNN(); break;
        case OP_FORCES: s.integrator.zeroStuff(); s.interactions.calcForces(); break;
        // the Green-strain / linear-C law of the reference's CPU path alone
        // (Interactions::calcFeaForcesCPU1, public, src/interactions.h:51)
        case OP_FEA_CPU1: s.integrator.zeroStuff(); s.interactions.calcFeaForcesCPU1(); break;
        case OP_DUMP_STATE: dump_state(s); break;
        case OP_DUMP_NN: dump_nn(s); break;
        case OP_DUMP_SETUP: dump_setup(s); break;
        case OP_SCALE: s.scale = rd<double>(); break;  // DukSystemSetScale (interface.cpp:365-369)
        case OP_SAVE: {
            // the writers print what the last property evaluation left: the
            // unfolded positions and centres of mass (calc_cluster_props,
            // interface.cpp:332-335) and v^2, as evalProps sets it
            // (md3dsystem.cpp:162-163; evalProps itself also adds to dispHi,
            // which would move the next list rebuild)
            int layout = rd<int32_t>(), append = rd<int32_t>(), n = rd<int32_t>();
            std::string name(n, '\0');
            if (n > 0 && fread(&name[0], 1, n, fin) != (size_t)n) { fprintf(stderr, "ref_harness: short name\n"); return 3; }
            std::string path = dir + "/" + name;
            if (!s.particles.feaElements.clusters.empty()) s.particles.feaElements.calcClusterProps();
            for (int i = 0; i < s.N; i++)
                s.particles.vv[i] = s.particles.vel[i].x * s.particles.vel[i].x + s.particles.vel[i].y * s.particles.vel[i].y;
            switch (layout) {
            case 0: s.saveClusterXYZ(path.c_str(), append); break;
            case 1: s.saveXYZ(path.c_str(), append); break;
            case 2: s.saveVtk(path.c_str()); break;
            case 3: s.saveVTF(path.c_str(), append); break;
            case 4: s.saveClusterVTF(path.c_str(), append); break;
            case 5: s.saveVtkXML(path.c_str()); break;
            case 6: s.saveVtkXMLBin(path.c_str()); break;
            default: fprintf(stderr, "ref_harness: unknown layout %d\n", layout); return 3;
            }
            break;
        }
        default: fprintf(stderr, "ref_harness: unknown op %d\n", op); return 3;
        }
    }
    wr<int32_t>(OP_END);
    fclose(fout);
    fclose(fin);
    return 0;
}
