// Host-side topology: the reference grid builder, input validation, and packing of
// many cloths into one ragged structure-of-arrays batch with a vertex->spring
// incidence (CSR) ordered by spring id.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "oc_internal.h"

namespace oc {
namespace {

inline int32_t float_bits(float f) {
    int32_t i;
    std::memcpy(&i, &f, sizeof(i));
    return i;
}

inline bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// splitmix64 (Steele, Lea, Flood 2014) and Box-Muller: a portable seeded normal stream.
inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double uniform_open01(uint64_t& s) { return ((double)(splitmix64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

}  // namespace

oc_status pack_instances(const oc_cloth_desc* descs, int32_t n, int32_t vpb, PackedHost* out, std::string* err) {
    if (!descs || n < 1 || !out || vpb < 1) {
        *err = "oc_create: descs must hold n_instances >= 1 cloths";
        return OC_ERR_INVALID_ARGUMENT;
    }
    int64_t nv = 0, ns = 0;
    bool any_ext = false;
    for (int32_t k = 0; k < n; ++k) {
        const oc_cloth_desc& d = descs[k];
        const std::string who = "instance " + std::to_string(k) + ": ";
        if (d.n_vertices < 1 || d.n_springs < 0 || (d.n_springs > 0 && !d.springs) || d.n_pinned < 0 ||
            (d.n_pinned > 0 && !d.pinned)) {
            *err = who + "bad sizes or NULL arrays";
            return OC_ERR_INVALID_ARGUMENT;
        }
        if (d.jacobian_mode != OC_JAC_REFERENCE && d.jacobian_mode != OC_JAC_COUPLED) {
            *err = who + "jacobian_mode " + std::to_string(d.jacobian_mode) + " is not available";
            return OC_ERR_UNSUPPORTED;
        }
        if (d.cg_max_iter < 0 || d.cg_max_iter > OC_MAX_CG_ITER || !std::isfinite(d.cg_tol) || d.cg_tol < 0.0f) {
            *err = who + "cg_max_iter must be in [0, OC_MAX_CG_ITER] and cg_tol finite and >= 0";
            return OC_ERR_INVALID_ARGUMENT;
        }
        if (!finite3(d.gravity) || !std::isfinite(d.velocity_damping)) {
            *err = who + "gravity / velocity_damping not finite";
            return OC_ERR_NON_FINITE;
        }
        for (int32_t s = 0; s < d.n_springs; ++s) {
            const oc_spring& sp = d.springs[s];
            if (sp.p1 < 0 || sp.p1 >= d.n_vertices || sp.p2 < 0 || sp.p2 >= d.n_vertices) {
                *err = who + "spring " + std::to_string(s) + " endpoint out of range";
                return OC_ERR_BAD_INDEX;
            }
            if (sp.p1 == sp.p2) {
                *err = who + "spring " + std::to_string(s) + " joins a vertex to itself";
                return OC_ERR_DEGENERATE;
            }
            if (!std::isfinite(sp.rest_length) || !std::isfinite(sp.ks) || !std::isfinite(sp.kd)) {
                *err = who + "spring " + std::to_string(s) + " has a non-finite parameter";
                return OC_ERR_NON_FINITE;
            }
            if (sp.rest_length < 0.0f) {
                *err = who + "spring " + std::to_string(s) + " has a negative rest length";
                return OC_ERR_INVALID_ARGUMENT;
            }
        }
        for (int32_t p = 0; p < d.n_pinned; ++p) {
            if (d.pinned[p] < 0 || d.pinned[p] >= d.n_vertices) {
                *err = who + "pinned index " + std::to_string(d.pinned[p]) + " out of range";
                return OC_ERR_BAD_INDEX;
            }
        }
        if (d.mass) {
            for (int32_t i = 0; i < d.n_vertices; ++i) {
                if (!std::isfinite(d.mass[i])) {
                    *err = who + "mass not finite";
                    return OC_ERR_NON_FINITE;
                }
                if (!(d.mass[i] > 0.0f)) {
                    *err = who + "mass must be > 0";
                    return OC_ERR_INVALID_ARGUMENT;
                }
            }
        }
        if (d.passes & ~(OC_PASS_ELLIPSOID | OC_PASS_PROVOT)) {
            *err = who + "unknown pass bits";
            return OC_ERR_INVALID_ARGUMENT;
        }
        if (d.passes & OC_PASS_ELLIPSOID) {
            for (int i = 0; i < 16; ++i) {
                if (!std::isfinite(d.ellipsoid[i]) || !std::isfinite(d.ellipsoid_inv[i])) {
                    *err = who + "ellipsoid matrix not finite";
                    return OC_ERR_NON_FINITE;
                }
            }
        }
        if ((d.passes & OC_PASS_PROVOT) && !(std::isfinite(d.provot_ratio) && d.provot_ratio >= 0.0f)) {
            *err = who + "provot_ratio must be finite and >= 0";
            return OC_ERR_INVALID_ARGUMENT;
        }
        if (d.ext_force) {
            any_ext = true;
            for (int32_t i = 0; i < d.n_vertices; ++i) {
                if (!finite3(d.ext_force + 3 * (size_t)i)) {
                    *err = who + "ext_force not finite";
                    return OC_ERR_NON_FINITE;
                }
            }
        }
        nv += d.n_vertices;
        ns += d.n_springs;
    }
    const int64_t int_max = std::numeric_limits<int32_t>::max();
    if (nv >= int_max || 2 * ns >= int_max) {
        *err = "batch too large: total vertices and 2 x total springs must stay below 2^31";
        return OC_ERR_UNSUPPORTED;
    }

    PackedHost& P = *out;
    P.n_inst = n;
    P.nv = nv;
    P.ns = ns;
    P.vertices_per_block = vpb;
    P.v_off.assign(n + 1, 0);
    P.s_off.assign(n + 1, 0);
    P.inst.resize(n);
    P.X0.assign(nv, make_float4(0.f, 0.f, 0.f, 1.f));
    P.V0.assign(nv, make_float4(0.f, 0.f, 0.f, 0.f));
    P.fext.clear();
    if (any_ext) P.fext.assign(nv, make_float4(0.f, 0.f, 0.f, 0.f));
    P.own_ends.assign(nv, make_int2(-1, -1));
    P.own_par.assign(nv, make_float4(0.f, 0.f, 0.f, 0.f));
    P.blocks.clear();
    P.any_provot = false;
    P.any_coupled = false;

    std::vector<int32_t> deg(nv, 0);
    for (int32_t k = 0; k < n; ++k) {
        const oc_cloth_desc& d = descs[k];
        P.v_off[k + 1] = P.v_off[k] + d.n_vertices;
        P.s_off[k + 1] = P.s_off[k] + d.n_springs;
        const int64_t vo = P.v_off[k];
        for (int32_t s = 0; s < d.n_springs; ++s) {
            ++deg[vo + d.springs[s].p1];
            ++deg[vo + d.springs[s].p2];
        }
    }
    P.rowptr.assign(nv + 1, 0);
    for (int64_t g = 0; g < nv; ++g) P.rowptr[g + 1] = P.rowptr[g] + deg[g];
    P.inc.assign((size_t)P.rowptr[nv], make_int4(0, 0, 0, 0));
    P.inc_sid.assign((size_t)P.rowptr[nv], 0);
    P.own_sid.assign(nv, -1);
    std::vector<int32_t> own_deg(nv, 0);
    std::vector<int32_t> cursor(P.rowptr.begin(), P.rowptr.end() - 1);

    for (int32_t k = 0; k < n; ++k) {
        const oc_cloth_desc& d = descs[k];
        const int64_t vo = P.v_off[k];
        InstParams& ip = P.inst[k];
        ip.gravity[0] = d.gravity[0];
        ip.gravity[1] = d.gravity[1];
        ip.gravity[2] = d.gravity[2];
        ip.damping = d.velocity_damping;
        const float eps = d.cg_tol;
        ip.eps2 = eps * eps;
        ip.imax = d.cg_max_iter;
        ip.v_off = vo;
        ip.nv = d.n_vertices;
        ip.has_ext = d.ext_force ? 1 : 0;
        ip.resident = 0;
        ip.passes = d.passes;
        ip.coupled = d.jacobian_mode == OC_JAC_COUPLED ? 1 : 0;
        if (ip.coupled) P.any_coupled = true;
        ip.provot_ratio = d.provot_ratio == 0.0f ? 1.01f : d.provot_ratio;
        for (int i = 0; i < 16; ++i) {
            ip.ellipsoid[i] = d.ellipsoid[i];
            ip.ellipsoid_inv[i] = d.ellipsoid_inv[i];
        }
        if (d.passes & OC_PASS_PROVOT) P.any_provot = true;
        ip.blk0 = (int32_t)P.blocks.size();
        ip.nblk = (d.n_vertices + vpb - 1) / vpb;
        for (int32_t b = 0; b < ip.nblk; ++b) {
            BlockInfo bi;
            bi.inst = k;
            bi.gblk = (int32_t)P.blocks.size();
            bi.v_begin = vo + (int64_t)b * vpb;
            bi.v_end = std::min<int64_t>(vo + d.n_vertices, bi.v_begin + vpb);
            P.blocks.push_back(bi);
        }
        for (int32_t i = 0; i < d.n_vertices; ++i) {
            P.X0[vo + i].w = d.mass ? d.mass[i] : 1.0f;
            if (d.ext_force)
                P.fext[vo + i] = make_float4(d.ext_force[3 * (size_t)i], d.ext_force[3 * (size_t)i + 1],
                                             d.ext_force[3 * (size_t)i + 2], 0.f);
        }
        for (int32_t p = 0; p < d.n_pinned; ++p) P.V0[vo + d.pinned[p]].w = 1.0f;
        for (int32_t s = 0; s < d.n_springs; ++s) {
            const oc_spring& sp = d.springs[s];
            const int32_t g1 = (int32_t)(vo + sp.p1), g2 = (int32_t)(vo + sp.p2);
            const int32_t rb = float_bits(sp.rest_length), kb = float_bits(sp.ks), db = float_bits(sp.kd);
            const int32_t sid = (int32_t)(P.s_off[k] + s);
            P.inc_sid[cursor[g1]] = sid;
            P.inc[cursor[g1]++] = make_int4(g2, rb, kb, db);
            P.inc_sid[cursor[g2]] = sid;
            P.inc[cursor[g2]++] = make_int4((int32_t)((uint32_t)g1 | 0x80000000u), rb, kb, db);
            if (s < d.n_vertices) {
                P.own_ends[vo + s] = make_int2(g1, g2);
                P.own_par[vo + s] = make_float4(sp.rest_length, sp.ks, sp.kd, 0.f);
                P.own_sid[vo + s] = sid;
                ++own_deg[g1];
                ++own_deg[g2];
            }
        }
    }
    // Grid cloths: the incidences of a vertex of a grid cloth made by the reference's
    // lattice (InitGL, IMP:497-565) depend only on its position class (first, second,
    // inner, third-last, second-last, last row, and the same for columns): the same neighbour offsets
    // in the same spring order, with parameters from a few distinct (rest, ks, kd).  Such
    // a cloth is stepped by a stencil kernel that reads no incidence records.  Every
    // vertex is checked against its class's template; any mismatch keeps the CSR path.
    P.st_data.clear();
    P.st_param.clear();
    P.any_st_rest = false;
    for (int32_t k = 0; k < n; ++k) {
        InstParams& ip = P.inst[k];
        ip.grid_cols = ip.grid_rows = 0;
        ip.st_off = ip.st_par = -1;
        ip.st_rest = 0;
        const int64_t vo = P.v_off[k];
        const int32_t nvk = ip.nv;
        if (nvk < 9) continue;
        int32_t cols = 0;
        for (int32_t e = P.rowptr[vo]; e < P.rowptr[vo + 1]; ++e) {
            const int32_t o = (int32_t)((P.inc[e].x & 0x7fffffff) - vo);
            if (o > 2 && (cols == 0 || o < cols)) cols = o;
        }
        if (cols < 3 || nvk % cols != 0 || nvk / cols < 3) continue;
        const int32_t rows = nvk / cols;
        // Two tries: parameter slots of (rest, ks, kd) -- no per-incidence data at all --
        // and, when the rest lengths vary (grid spacings that FP32 does not hold exactly),
        // slots of (ks, kd) with the rest lengths read per incidence.
        std::vector<int4> slots;  // rest, ks, kd bits
        std::vector<std::vector<int32_t>> tmpl;
        bool ok = false;
        int32_t mode = 0;
        for (int32_t try_mode = 1; try_mode <= 2 && !ok; ++try_mode) {
            const bool with_rest = try_mode == 1;
            slots.clear();
            tmpl.assign(kStencilClasses, std::vector<int32_t>());
            std::vector<int32_t> rep(kStencilClasses, -1);
            ok = true;
            auto entry_of = [&](int32_t l, int32_t e, int32_t* out) -> bool {
                const int4 rec = P.inc[e];
                const int32_t o = (int32_t)((rec.x & 0x7fffffff) - vo);
                const int32_t r = l / cols, c = l % cols, ro = o / cols, co = o % cols;
                const int32_t di = ro - r, dj = co - c;
                if (o < 0 || o >= nvk || di < -2 || di > 2 || dj < -2 || dj > 2) return false;
                const int32_t rest_key = with_rest ? rec.y : 0;
                int32_t slot = -1;
                for (size_t q = 0; q < slots.size(); ++q)
                    if (slots[q].y == rest_key && slots[q].z == rec.z && slots[q].w == rec.w) slot = (int32_t)q;
                if (slot < 0) {
                    if ((int)slots.size() >= kStencilSlots) return false;
                    slot = (int32_t)slots.size();
                    slots.push_back(make_int4(0, rest_key, rec.z, rec.w));
                }
                *out = (di + 2) | ((dj + 2) << 3) | ((rec.x < 0 ? 1 : 0) << 6) | (slot << 7);
                return true;
            };
            // Templates from the first vertex of each class.
            for (int32_t l = 0; l < nvk && ok; ++l) {
                const int cl = stencil_class_1d(l / cols, rows) * 6 + stencil_class_1d(l % cols, cols);
                if (rep[cl] >= 0) continue;
                rep[cl] = l;
                for (int32_t e = P.rowptr[vo + l]; e < P.rowptr[vo + l + 1] && ok; ++e) {
                    int32_t v = 0;
                    ok = entry_of(l, e, &v);
                    tmpl[cl].push_back(v);
                }
            }
            // Every vertex against its template.
            for (int32_t l = 0; l < nvk && ok; ++l) {
                const int cl = stencil_class_1d(l / cols, rows) * 6 + stencil_class_1d(l % cols, cols);
                const int32_t e0 = P.rowptr[vo + l], e1 = P.rowptr[vo + l + 1];
                if ((size_t)(e1 - e0) != tmpl[cl].size()) ok = false;
                for (int32_t e = e0; e < e1 && ok; ++e) {
                    int32_t v = 0;
                    ok = entry_of(l, e, &v) && v == tmpl[cl][e - e0];
                }
            }
            if (ok) mode = try_mode;
        }
        if (!ok) continue;
        ip.st_rest = mode == 2 ? 1 : 0;
        if (mode == 2) P.any_st_rest = true;
        ip.grid_cols = cols;
        ip.grid_rows = rows;
        ip.st_off = (int32_t)P.st_data.size();
        int32_t pos = kStencilClasses + 1;
        for (int cl = 0; cl < kStencilClasses; ++cl) {
            P.st_data.push_back(pos);
            pos += (int32_t)tmpl[cl].size();
        }
        P.st_data.push_back(pos);
        for (int cl = 0; cl < kStencilClasses; ++cl) P.st_data.insert(P.st_data.end(), tmpl[cl].begin(), tmpl[cl].end());
        ip.st_par = (int32_t)P.st_param.size();
        for (int q = 0; q < kStencilSlots; ++q) {
            float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q < (int)slots.size()) {
                std::memcpy(&f.x, &slots[q].y, 4);
                std::memcpy(&f.y, &slots[q].z, 4);
                std::memcpy(&f.z, &slots[q].w, 4);
            }
            P.st_param.push_back(f);
        }
    }
    // Vertex -> vertices whose own spring (spring i for vertex i) touches it, ordered by i.
    P.own_rowptr.assign(nv + 1, 0);
    for (int64_t g = 0; g < nv; ++g) P.own_rowptr[g + 1] = P.own_rowptr[g] + own_deg[g];
    P.own_ent.assign((size_t)P.own_rowptr[nv], 0);
    std::vector<int32_t> oc(P.own_rowptr.begin(), P.own_rowptr.end() - 1);
    for (int64_t i = 0; i < nv; ++i) {
        const int2 e = P.own_ends[i];
        if (e.x < 0) continue;
        P.own_ent[oc[e.x]++] = (int32_t)i;
        P.own_ent[oc[e.y]++] = (int32_t)((uint32_t)i | 0x80000000u);
    }
    return OC_OK;
}

// The strip sweep's tables.  A grid cloth qualifies when every vertex's incidences are,
// in order, the springs the reference's InitGL loops give it (IMP:531-565), listed below
// with the anchor that owns each spring in the sweep (the spring's upper-left end; for
// the second shear spring of a quad, the quad's upper-left corner), and every spring of a
// kind whose anchor lies in one position class shares one parameter slot.  The repeated
// bend springs of the last three rows and columns must share their original's slot (and
// rest length), so the sweep reuses the original's force for them.
namespace {

enum StripKind { SK_H = 0, SK_BR = 1, SK_V = 2, SK_SHA = 3, SK_SHB = 4, SK_BC = 5 };

struct StripEntry {
    int8_t dr, dc, p2, kind;
    int32_t ar, ac;  // anchor
};

// Vertex (r, c)'s incidences in spring-id order (the kernel adds them in this order).
int strip_entries(int32_t r, int32_t c, int32_t rows, int32_t cols, StripEntry* out) {
    int n = 0;
    auto add = [&](int dr, int dc, int p2, int kind, int32_t ar, int32_t ac) {
        out[n++] = StripEntry{(int8_t)dr, (int8_t)dc, (int8_t)p2, (int8_t)kind, ar, ac};
    };
    if (c >= 1) add(0, -1, 1, SK_H, r, c - 1);                                    // horizontal structural
    if (c + 1 < cols) add(0, 1, 0, SK_H, r, c);
    if (r >= 1) add(-1, 0, 1, SK_V, r - 1, c);                                    // vertical structural
    if (r + 1 < rows) add(1, 0, 0, SK_V, r, c);
    if (r >= 1 && c >= 1) add(-1, -1, 1, SK_SHA, r - 1, c - 1);                   // shear, quad by quad
    if (r >= 1 && c + 1 < cols) add(-1, 1, 0, SK_SHB, r - 1, c);
    if (r + 1 < rows && c >= 1) add(1, -1, 1, SK_SHB, r, c - 1);
    if (r + 1 < rows && c + 1 < cols) add(1, 1, 0, SK_SHA, r, c);
    if (c >= 2) add(0, -2, 1, SK_BR, r, c - 2);                                   // bend along the row
    if (c + 2 < cols) add(0, 2, 0, SK_BR, r, c);
    if (c == cols - 3) add(0, 2, 0, SK_BR, r, c);                                 // its repeat
    if (c == cols - 1) add(0, -2, 1, SK_BR, r, c - 2);
    if (r >= 2) add(-2, 0, 1, SK_BC, r - 2, c);                                   // bend along the column
    if (r + 2 < rows) add(2, 0, 0, SK_BC, r, c);
    if (r == rows - 3) add(2, 0, 0, SK_BC, r, c);                                 // its repeat
    if (r == rows - 1) add(-2, 0, 1, SK_BC, r - 2, c);
    return n;
}

}  // namespace

void build_strip_tables(PackedHost* Pp) {
    PackedHost& P = *Pp;
    P.strip_slot.clear();
    P.strip_rest.clear();
    for (int32_t k = 0; k < P.n_inst; ++k) {
        InstParams& ip = P.inst[k];
        ip.strip = ip.strip_ok = 0;
        ip.strip_slot = -1;
        ip.strip_rest = -1;
        if (ip.grid_cols <= 0 || ip.coupled) continue;
        const int32_t cols = ip.grid_cols, rows = ip.grid_rows, nvk = ip.nv;
        const int64_t vo = P.v_off[k];
        const int32_t* st = P.st_data.data() + ip.st_off;
        int slot[6][kStencilClasses];
        for (auto& row : slot)
            for (int& x : row) x = -1;
        std::vector<int32_t> rest_bits(ip.st_rest ? 6 * (size_t)nvk : 0, 0);
        std::vector<uint8_t> rest_set(rest_bits.size(), 0);
        bool ok = true;
        StripEntry ex[16];
        for (int32_t l = 0; l < nvk && ok; ++l) {
            const int32_t r = l / cols, c = l % cols;
            const int cl = stencil_class_1d(r, rows) * 6 + stencil_class_1d(c, cols);
            const int32_t e0 = st[cl], e1 = st[cl + 1];
            const int n = strip_entries(r, c, rows, cols, ex);
            if (n != e1 - e0) {
                ok = false;
                break;
            }
            for (int i = 0; i < n && ok; ++i) {
                const int32_t v = st[e0 + i];
                if ((v & 7) - 2 != ex[i].dr || ((v >> 3) & 7) - 2 != ex[i].dc || ((v >> 6) & 1) != ex[i].p2) {
                    ok = false;
                    break;
                }
                const int acl = stencil_class_1d(ex[i].ar, rows) * 6 + stencil_class_1d(ex[i].ac, cols);
                int& sl = slot[ex[i].kind][acl];
                if (sl < 0)
                    sl = v >> 7;
                else if (sl != (v >> 7))
                    ok = false;
                if (ip.st_rest && ok) {
                    const size_t at = (size_t)ex[i].kind * nvk + (size_t)ex[i].ar * cols + ex[i].ac;
                    const int32_t rb = P.inc[(size_t)(P.rowptr[vo + l] + i)].y;
                    if (!rest_set[at]) {
                        rest_set[at] = 1;
                        rest_bits[at] = rb;
                    } else if (rest_bits[at] != rb) {
                        ok = false;
                    }
                }
            }
        }
        if (!ok) continue;
        ip.strip_ok = 1;
        ip.strip_slot = (int32_t)P.strip_slot.size();
        for (int cl = 0; cl < kStencilClasses; ++cl) {
            uint32_t w = 0;
            for (int kind = 0; kind < 6; ++kind) w |= (uint32_t)(std::max(slot[kind][cl], 0) & 15) << (4 * kind);
            P.strip_slot.push_back(w);
        }
        if (ip.st_rest) {
            ip.strip_rest = (int64_t)P.strip_rest.size();
            const size_t base = P.strip_rest.size();
            P.strip_rest.resize(base + rest_bits.size());
            std::memcpy(P.strip_rest.data() + base, rest_bits.data(), rest_bits.size() * sizeof(float));
        }
    }
}

}  // namespace oc

extern "C" {

oc_status oc_describe_instances(const oc_cloth_desc* descs, int32_t n_instances, int32_t* grid_cols,
                                int32_t* grid_rows) {
    if (!descs || n_instances < 1) return OC_ERR_INVALID_ARGUMENT;
    oc::PackedHost P;
    std::string err;
    const oc_status st = oc::pack_instances(descs, n_instances, 2048, &P, &err);
    if (st != OC_OK) return st;
    for (int32_t k = 0; k < n_instances; ++k) {
        if (grid_cols) grid_cols[k] = P.inst[k].grid_cols;
        if (grid_rows) grid_rows[k] = P.inst[k].grid_rows;
    }
    return OC_OK;
}

oc_status oc_grid_spring_count(int32_t cols, int32_t rows, int32_t* n_springs) {
    if (!n_springs || cols < 3 || rows < 3) return OC_ERR_INVALID_ARGUMENT;
    const int64_t u = cols, v = rows;
    const int64_t s = v * (u - 1) + u * (v - 1) + 2 * (v - 1) * (u - 1) + v * (u - 1) + u * (v - 1);
    if (s >= std::numeric_limits<int32_t>::max()) return OC_ERR_UNSUPPORTED;
    *n_springs = (int32_t)s;
    return OC_OK;
}

// Mirrors InitGL's lattice and spring loops, IMP:497-565 (AddSpring IMP:370-380 takes
// the rest length from the positions at creation, before any jitter).
oc_status oc_grid_build(int32_t cols, int32_t rows, float size, const float ks[3], const float kd[3], float jitter,
                        uint64_t seed, float* X, oc_spring* springs) {
    int32_t ns = 0;
    if (oc_grid_spring_count(cols, rows, &ns) != OC_OK || !ks || !kd || !X || !springs ||
        !(size > 0.0f) || !std::isfinite(size) || !std::isfinite(jitter) || jitter < 0.0f)
        return OC_ERR_INVALID_ARGUMENT;
    const int32_t u = cols, v = rows;
    const float halfsize = size / 2.0f;
    for (int32_t j = 0; j < v; ++j) {
        for (int32_t i = 0; i < u; ++i) {
            float* p = X + 3 * ((size_t)j * u + i);
            p[0] = (((float)i / (float)(u - 1)) * 2.0f - 1.0f) * halfsize;
            p[1] = (size + 1.0f) - ((float)j / (float)(v - 1)) * size;
            p[2] = 0.0f;
        }
    }
    int32_t c = 0;
    auto add = [&](int32_t a, int32_t b, int32_t type) {
        oc_spring& sp = springs[c++];
        sp.p1 = a;
        sp.p2 = b;
        sp.ks = ks[type];
        sp.kd = kd[type];
        sp.type = type;
        const float dx = X[3 * (size_t)a] - X[3 * (size_t)b];
        const float dy = X[3 * (size_t)a + 1] - X[3 * (size_t)b + 1];
        const float dz = X[3 * (size_t)a + 2] - X[3 * (size_t)b + 2];
        sp.rest_length = std::sqrt(dx * dx + dy * dy + dz * dz);
    };
    for (int32_t l1 = 0; l1 < v; ++l1)  // horizontal structural
        for (int32_t l2 = 0; l2 < u - 1; ++l2) add(l1 * u + l2, l1 * u + l2 + 1, OC_STRUCTURAL_SPRING);
    for (int32_t l1 = 0; l1 < u; ++l1)  // vertical structural
        for (int32_t l2 = 0; l2 < v - 1; ++l2) add(l2 * u + l1, (l2 + 1) * u + l1, OC_STRUCTURAL_SPRING);
    for (int32_t l1 = 0; l1 < v - 1; ++l1)  // shear, two per quad
        for (int32_t l2 = 0; l2 < u - 1; ++l2) {
            add(l1 * u + l2, (l1 + 1) * u + l2 + 1, OC_SHEAR_SPRING);
            add((l1 + 1) * u + l2, l1 * u + l2 + 1, OC_SHEAR_SPRING);
        }
    for (int32_t l1 = 0; l1 < v; ++l1) {  // bend along rows, plus the reference's repeat of the last one
        for (int32_t l2 = 0; l2 < u - 2; ++l2) add(l1 * u + l2, l1 * u + l2 + 2, OC_BEND_SPRING);
        add(l1 * u + (u - 3), l1 * u + (u - 1), OC_BEND_SPRING);
    }
    for (int32_t l1 = 0; l1 < u; ++l1) {  // bend along columns, same repeat
        for (int32_t l2 = 0; l2 < v - 2; ++l2) add(l2 * u + l1, (l2 + 2) * u + l1, OC_BEND_SPRING);
        add((v - 3) * u + l1, (v - 1) * u + l1, OC_BEND_SPRING);
    }
    if (jitter > 0.0f) {
        const double sigma = (double)jitter * (double)size / (double)(u - 1);
        uint64_t state = seed;
        const size_t n3 = 3 * (size_t)u * v;
        for (size_t k = 0; k < n3; k += 2) {
            const double r = std::sqrt(-2.0 * std::log(oc::uniform_open01(state)));
            const double t = 6.283185307179586 * oc::uniform_open01(state);
            X[k] += (float)(sigma * r * std::cos(t));
            if (k + 1 < n3) X[k + 1] += (float)(sigma * r * std::sin(t));
        }
    }
    return c == ns ? OC_OK : OC_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
