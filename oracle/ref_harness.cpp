// Test infrastructure (oracle only; never linked into the library).
//
// Headless driver for the reference's own implicit step.  It #includes a generated
// copy of OpenCloth_Implicit/OpenCloth_Implicit/main.cpp (made by build_ref.sh, which
// only turns the grid size IMP:60 and the CG constants IMP:126/128 into run-time
// values) and calls the reference's functions unchanged:
//
//   InitGL()                      main.cpp:468  (arrays, reference springs)
//   ComputeForces()               main.cpp:698
//   IntegrateImplicit(dt)         main.cpp:775  (CalcForceDerivatives + PCG + update)
//
// Inputs (positions, velocities, warm-start dV, springs, gravity) come from an
// instance file and overwrite the globals InitGL() set up, so any grid-shaped cloth
// (pins at the reference's hard-coded indices 0 and numX) can be stepped.
//
// Build flavours: OC_REAL=float (the reference as written) or OC_REAL=double (the
// same source with glm vec/mat -> dvec/dmat and float -> double).
//
// Usage:
//   ref_step <instance.bin> <out.bin> [--time]   step and write snapshots
//   ref_step --topology <out.bin>                dump InitGL()'s springs and X
//   ref_step --ellipsoid <out.bin>               dump InitGL()'s ellipsoid matrices
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static int oc_env_int(const char* key, int fallback) {
    const char* s = std::getenv(key);
    return s ? std::atoi(s) : fallback;
}
static double oc_env_real(const char* key, double fallback) {
    const char* s = std::getenv(key);
    return s ? std::strtod(s, nullptr) : fallback;
}

#define main ref_main
#include OC_REF_SOURCE
#undef main

typedef OC_REAL real_t;

namespace {

struct InstanceHeader {
    char magic[4];
    int32_t n_vertices, n_springs, num_x, num_y, i_max;
    float eps, dt, gravity[3];
    int32_t n_snap;
};

struct SpringRecord {
    int32_t p1, p2;
    float rest, ks, kd;
    int32_t type;
};

bool read_exact(FILE* f, void* dst, size_t bytes) { return std::fread(dst, 1, bytes, f) == bytes; }

void write_state(FILE* f, int32_t step) {
    std::fwrite(&step, sizeof(step), 1, f);
    const size_t n = total_points;
    std::vector<real_t> buf(3 * n);
    for (size_t i = 0; i < n; ++i) { buf[3 * i] = X[i].x; buf[3 * i + 1] = X[i].y; buf[3 * i + 2] = X[i].z; }
    std::fwrite(buf.data(), sizeof(real_t), buf.size(), f);
    for (size_t i = 0; i < n; ++i) { buf[3 * i] = V[i].x; buf[3 * i + 1] = V[i].y; buf[3 * i + 2] = V[i].z; }
    std::fwrite(buf.data(), sizeof(real_t), buf.size(), f);
    for (size_t i = 0; i < n; ++i) { buf[3 * i] = dV[i].x; buf[3 * i + 1] = dV[i].y; buf[3 * i + 2] = dV[i].z; }
    std::fwrite(buf.data(), sizeof(real_t), buf.size(), f);
}

int dump_topology(const char* out_path) {
    InitGL();
    FILE* f = std::fopen(out_path, "wb");
    if (!f) return 2;
    int32_t hdr[2] = {(int32_t)total_points, (int32_t)springs.size()};
    std::fwrite(hdr, sizeof(hdr), 1, f);
    for (size_t i = 0; i < total_points; ++i) {
        real_t p[3] = {X[i].x, X[i].y, X[i].z};
        std::fwrite(p, sizeof(real_t), 3, f);
    }
    for (size_t s = 0; s < springs.size(); ++s) {
        SpringRecord r;
        r.p1 = springs[s].p1;
        r.p2 = springs[s].p2;
        r.rest = (float)springs[s].rest_length;
        r.ks = (float)springs[s].Ks;
        r.kd = (float)springs[s].Kd;
        r.type = springs[s].type;
        std::fwrite(&r, sizeof(r), 1, f);
    }
    std::fclose(f);
    return 0;
}

}  // namespace

// The reference's ellipsoid (InitGL, IMP:583-586): the object-to-world matrix and its
// inverse, 16 reals each (float or double with the build), glm column-major.
int dump_ellipsoid(const char* out_path) {
    InitGL();
    FILE* f = std::fopen(out_path, "wb");
    if (!f) return 2;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            const real_t v = ellipsoid[c][r];
            std::fwrite(&v, sizeof(v), 1, f);
        }
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            const real_t v = inverse_ellipsoid[c][r];
            std::fwrite(&v, sizeof(v), 1, f);
        }
    std::fclose(f);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 3 && std::string(argv[1]) == "--topology") return dump_topology(argv[2]);
    if (argc >= 3 && std::string(argv[1]) == "--ellipsoid") return dump_ellipsoid(argv[2]);
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <instance.bin> <out.bin> [--time] | --topology <out.bin>\n", argv[0]);
        return 2;
    }
    const bool timed = argc >= 4 && std::string(argv[3]) == "--time";
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", argv[1]); return 2; }
    InstanceHeader h;
    if (!read_exact(f, &h, sizeof(h)) || std::memcmp(h.magic, "OCI1", 4) != 0) {
        std::fprintf(stderr, "bad instance header\n");
        return 2;
    }
    // The grid size and CG constants are compile-time constants in the reference; the
    // generated copy reads them from the environment at start-up.  They must agree.
    if (h.num_x != numX || h.num_y != numY || (size_t)h.n_vertices != total_points || h.i_max != i_max ||
        (float)h.eps != (float)EPS) {
        std::fprintf(stderr, "instance/env mismatch: numX %d/%d numY %d/%d N %d/%zu imax %d/%d\n", h.num_x, numX,
                     h.num_y, numY, h.n_vertices, (size_t)total_points, h.i_max, i_max);
        return 3;
    }
    std::vector<int32_t> snaps(h.n_snap);
    std::vector<float> x0(3 * (size_t)h.n_vertices), v0(x0.size()), dv0(x0.size());
    std::vector<SpringRecord> recs(h.n_springs);
    bool ok = read_exact(f, snaps.data(), sizeof(int32_t) * snaps.size()) &&
              read_exact(f, x0.data(), sizeof(float) * x0.size()) &&
              read_exact(f, v0.data(), sizeof(float) * v0.size()) &&
              read_exact(f, dv0.data(), sizeof(float) * dv0.size()) &&
              read_exact(f, recs.data(), sizeof(SpringRecord) * recs.size());
    std::fclose(f);
    if (!ok) { std::fprintf(stderr, "truncated instance\n"); return 2; }

    InitGL();
    gravity.x = h.gravity[0];
    gravity.y = h.gravity[1];
    gravity.z = h.gravity[2];

    springs.clear();
    for (const SpringRecord& r : recs) {
        decltype(springs)::value_type sp;
        sp.p1 = r.p1;
        sp.p2 = r.p2;
        sp.rest_length = r.rest;
        sp.Ks = r.ks;
        sp.Kd = r.kd;
        sp.type = r.type;
        springs.push_back(sp);
    }
    // Per-spring scratch, sized and cleared as InitGL() does (main.cpp:567-577).
    const size_t S = springs.size();
    C.assign(S, 0);
    inv_len.assign(S, 0);
    C_Dot.assign(S, 0);
    dc_dp.assign(S, decltype(dc_dp)::value_type(0));
    deltaP2.assign(S, decltype(deltaP2)::value_type(0));
    df_dx.assign(S, decltype(df_dx)::value_type(0));
    df_dv.assign(S, decltype(df_dv)::value_type(0));

    for (size_t i = 0; i < total_points; ++i) {
        X[i].x = x0[3 * i]; X[i].y = x0[3 * i + 1]; X[i].z = x0[3 * i + 2];
        V[i].x = v0[3 * i]; V[i].y = v0[3 * i + 1]; V[i].z = v0[3 * i + 2];
        dV[i].x = dv0[3 * i]; dV[i].y = dv0[3 * i + 1]; dV[i].z = dv0[3 * i + 2];
    }

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    std::fwrite("OCO1", 1, 4, out);
    int32_t real_size = sizeof(real_t);
    std::fwrite(&real_size, sizeof(real_size), 1, out);
    std::fwrite(&h.n_snap, sizeof(h.n_snap), 1, out);

    const int32_t last = snaps.empty() ? 0 : snaps.back();
    size_t next = 0;
    while (next < snaps.size() && snaps[next] == 0) write_state(out, 0), ++next;
    const real_t dt = h.dt;
    auto t0 = std::chrono::steady_clock::now();
    // OC_PASSES bit 1: EllipsoidCollision (IMP:824), bit 2: ApplyProvotDynamicInverse
    // (IMP:800), in StepPhysics' order (IMP:873-880).
    const int passes = oc_env_int("OC_PASSES", 0);
    for (int32_t step = 1; step <= last; ++step) {
        ComputeForces();
        IntegrateImplicit(dt);
        if (passes & 1) EllipsoidCollision();
        if (passes & 2) ApplyProvotDynamicInverse();
        while (next < snaps.size() && snaps[next] == step) write_state(out, step), ++next;
    }
    auto t1 = std::chrono::steady_clock::now();
    std::fclose(out);
    if (timed) {
        double s = std::chrono::duration<double>(t1 - t0).count();
        std::printf("{\"steps\": %d, \"seconds\": %.6f, \"vertices\": %zu}\n", last, s, (size_t)total_points);
    }
    return 0;
}
