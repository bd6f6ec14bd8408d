// Test infrastructure (oracle only; never linked into the library).
//
// Headless driver for the reference's co-rotated linear FEM demo,
// OpenCloth_CoRotated_Linear_FEM/OpenCloth_CoRotated_Linear_FEM/main.cpp (FEM).  It
// #includes a generated copy of that file (made by build_ref.sh, which only turns the
// mesh size of InitGL, FEM:425, into run-time values) and calls the reference's
// functions unchanged:
//
//   InitGL()                   FEM:424   mesh, element stiffness, lumped masses
//   StepPhysics(dt)            FEM:981   whole steps, to reach a deformed state
//   ComputeForces ... DynamicsAssembly   FEM:983-995, the first half of one more step
//   ConjugateGradientSolver    FEM:837-922, the block-sparse CG the library restates
//
// Usage:
//   fem_step --system <steps> <system.bin> <solution.bin>
//       InitGL, `steps` steps, then the assembly of one more step: writes the system the
//       CG receives and the CG's own result.
//   fem_step --solve <system.bin> <solution.bin> [--time]
//       the reference CG on a stored system.
//
// System file: "OCB1", int32 n, nnzb, i_max; float tolerance, tiny; int32 row_ptr[n+1],
// col[nnzb] (ascending within a row, std::map's order); float blocks[9 nnzb] (m[c][r]
// at 3c + r, glm's layout); float b[3n], V[3n] (warm start); uint8 fixed[n].
// Solution file: real V[3n] then residual[3n] (real = float or double with the build).
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

#define main ref_main
#include OC_FEM_SOURCE
#undef main

typedef OC_REAL real_t;

namespace {

bool read_exact(FILE* f, void* dst, size_t bytes) { return std::fread(dst, 1, bytes, f) == bytes; }

struct Header {
    char magic[4];
    int32_t n, nnzb, i_max;
    float tol, tiny;
};

void write_solution(const char* path) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return;
    std::vector<real_t> buf(3 * total_points);
    for (size_t i = 0; i < total_points; ++i) { buf[3 * i] = V[i].x; buf[3 * i + 1] = V[i].y; buf[3 * i + 2] = V[i].z; }
    std::fwrite(buf.data(), sizeof(real_t), buf.size(), f);
    for (size_t i = 0; i < total_points; ++i) {
        buf[3 * i] = residual[i].x; buf[3 * i + 1] = residual[i].y; buf[3 * i + 2] = residual[i].z;
    }
    std::fwrite(buf.data(), sizeof(real_t), buf.size(), f);
    std::fclose(f);
}

int dump_system(const char* path) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return 2;
    Header h;
    std::memcpy(h.magic, "OCB1", 4);
    h.n = (int32_t)total_points;
    std::vector<int32_t> row_ptr(1, 0), col;
    std::vector<float> blocks;
    for (size_t k = 0; k < total_points; ++k) {
        for (matrix_iterator it = A_row[k].begin(); it != A_row[k].end(); ++it) {
            col.push_back((int32_t)it->first);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) blocks.push_back((float)it->second[c][r]);
        }
        row_ptr.push_back((int32_t)col.size());
    }
    h.nnzb = (int32_t)col.size();
    h.i_max = i_max;
    h.tol = (float)tolerence;
    h.tiny = (float)tiny;
    std::fwrite(&h, sizeof(h), 1, f);
    std::fwrite(row_ptr.data(), sizeof(int32_t), row_ptr.size(), f);
    std::fwrite(col.data(), sizeof(int32_t), col.size(), f);
    std::fwrite(blocks.data(), sizeof(float), blocks.size(), f);
    std::vector<float> v(3 * total_points);
    for (size_t i = 0; i < total_points; ++i) { v[3 * i] = (float)b[i].x; v[3 * i + 1] = (float)b[i].y; v[3 * i + 2] = (float)b[i].z; }
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    for (size_t i = 0; i < total_points; ++i) { v[3 * i] = (float)V[i].x; v[3 * i + 1] = (float)V[i].y; v[3 * i + 2] = (float)V[i].z; }
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    for (size_t i = 0; i < total_points; ++i) {
        const uint8_t fx = IsFixed[i] ? 1 : 0;
        std::fwrite(&fx, 1, 1, f);
    }
    std::fclose(f);
    return 0;
}

int run_system(int steps, const char* sys_path, const char* sol_path) {
    InitGL();
    for (int s = 0; s < steps; ++s) StepPhysics(timeStep);
    // StepPhysics (FEM:981-1000) up to the solve.
    const float dt = timeStep;
    ComputeForces();
    ClearStiffnessAssembly();
    if (bUseStiffnessWarping)
        UpdateOrientation();
    else
        ResetOrientation();
    StiffnessAssembly();
    AddPlasticityForce(dt);
    DynamicsAssembly(dt);
    if (int e = dump_system(sys_path)) return e;
    ConjugateGradientSolver(dt);
    write_solution(sol_path);
    return 0;
}

int run_solve(const char* sys_path, const char* sol_path, bool timed) {
    FILE* f = std::fopen(sys_path, "rb");
    if (!f) return 2;
    Header h;
    if (!read_exact(f, &h, sizeof(h)) || std::memcmp(h.magic, "OCB1", 4) != 0 || h.n < 1 || h.nnzb < 0) {
        std::fclose(f);
        return 2;
    }
    std::vector<int32_t> row_ptr(h.n + 1), col(h.nnzb);
    std::vector<float> blocks(9 * (size_t)h.nnzb), bb(3 * (size_t)h.n), vv(3 * (size_t)h.n);
    std::vector<uint8_t> fixed(h.n);
    bool ok = read_exact(f, row_ptr.data(), 4 * row_ptr.size()) && read_exact(f, col.data(), 4 * col.size()) &&
              read_exact(f, blocks.data(), 4 * blocks.size()) && read_exact(f, bb.data(), 4 * bb.size()) &&
              read_exact(f, vv.data(), 4 * vv.size()) && read_exact(f, fixed.data(), fixed.size());
    std::fclose(f);
    if (!ok) return 2;
    // The globals ConjugateGradientSolver reads, sized and zeroed as InitGL leaves them
    // (FEM:430-441); `previous` of a fixed vertex is never written and stays zero.
    typedef decltype(b)::value_type vec_t;
    typedef matrix_map::mapped_type mat_t;
    total_points = (size_t)h.n;
    A_row.assign(total_points, matrix_map());
    b.assign(total_points, vec_t(0));
    V.assign(total_points, vec_t(0));
    residual.assign(total_points, vec_t(0));
    previous.assign(total_points, vec_t(0));
    update.assign(total_points, vec_t(0));
    IsFixed.assign(total_points, false);
    for (int32_t k = 0; k < h.n; ++k) {
        for (int32_t e = row_ptr[k]; e < row_ptr[k + 1]; ++e) {
            mat_t m;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) m[c][r] = blocks[9 * (size_t)e + 3 * c + r];
            A_row[k][col[e]] = m;
        }
        b[k] = vec_t(bb[3 * k], bb[3 * k + 1], bb[3 * k + 2]);
        V[k] = vec_t(vv[3 * k], vv[3 * k + 1], vv[3 * k + 2]);
        IsFixed[k] = fixed[k] != 0;
    }
    i_max = h.i_max;
    tolerence = h.tol;
    tiny = h.tiny;
    auto t0 = std::chrono::steady_clock::now();
    ConjugateGradientSolver(timeStep);
    auto t1 = std::chrono::steady_clock::now();
    write_solution(sol_path);
    if (timed)
        std::printf("{\"seconds\": %.6f, \"rows\": %d, \"nnzb\": %d}\n", std::chrono::duration<double>(t1 - t0).count(),
                    h.n, h.nnzb);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 5 && std::string(argv[1]) == "--system") return run_system(std::atoi(argv[2]), argv[3], argv[4]);
    if (argc >= 4 && std::string(argv[1]) == "--solve")
        return run_solve(argv[2], argv[3], argc >= 5 && std::string(argv[4]) == "--time");
    std::fprintf(stderr, "usage: %s --system <steps> <system.bin> <solution.bin> | --solve <system.bin> <solution.bin>\n",
                 argv[0]);
    return 2;
}
