// Host side of triangle-mesh boundary objects: OBJ parsing, pseudonormals, BVH construction.
#include "vfs_mesh.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <unordered_map>

namespace vfs {

namespace {

struct V3 {
    float x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 a) {
    const float l = std::sqrt(dot(a, a));
    return mul(1.0f / l, a);
}

// Index of an OBJ face corner "v", "v/t", "v//n" or "v/t/n" (1-based, negative = relative).
bool corner_index(const char* tok, long n_vertices, long& out) {
    char* end = nullptr;
    const long v = std::strtol(tok, &end, 10);
    if (end == tok || v == 0) return false;
    out = v > 0 ? v - 1 : n_vertices + v;
    return out >= 0 && out < n_vertices;
}

}  // namespace

bool load_obj(const std::string& path, std::vector<float>& pos, std::vector<uint32_t>& tri,
              std::string& err) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) {
        err = "cannot read " + path;
        return false;
    }
    std::vector<float> all;  // every "v" of the file (OBJ indices are file-global)
    std::vector<long> faces;  // global vertex index per corner of the current object's triangles
    std::vector<long> last_faces;
    bool in_object_with_faces = false;
    char line[4096];
    long lineno = 0;
    bool ok = true;
    while (ok && std::fgets(line, sizeof(line), f)) {
        lineno++;
        char* s = line;
        while (*s == ' ' || *s == '\t') s++;
        if ((s[0] == 'o' || s[0] == 'g') && (s[1] == ' ' || s[1] == '\t' || s[1] == '\n')) {
            // A new object: LoadObjMesh keeps one mesh per shape and the scene takes the last.
            if (!faces.empty()) {
                last_faces.swap(faces);
                faces.clear();
            }
            in_object_with_faces = false;
        } else if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
            float x, y, z;
            if (std::sscanf(s + 1, "%f %f %f", &x, &y, &z) != 3) {
                err = path + ":" + std::to_string(lineno) + ": bad vertex";
                ok = false;
                break;
            }
            all.insert(all.end(), {x, y, z});
        } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
            std::vector<long> poly;
            char* tok = std::strtok(s + 1, " \t\r\n");
            while (tok) {
                long idx;
                if (!corner_index(tok, (long)(all.size() / 3), idx)) {
                    err = path + ":" + std::to_string(lineno) + ": bad face index";
                    ok = false;
                    break;
                }
                poly.push_back(idx);
                tok = std::strtok(nullptr, " \t\r\n");
            }
            if (!ok) break;
            if (poly.size() < 3) {
                err = path + ":" + std::to_string(lineno) + ": face with fewer than 3 corners";
                ok = false;
                break;
            }
            for (size_t k = 1; k + 1 < poly.size(); k++) faces.insert(faces.end(), {poly[0], poly[k], poly[k + 1]});
            in_object_with_faces = true;
        }
    }
    std::fclose(f);
    if (!ok) return false;
    (void)in_object_with_faces;
    const std::vector<long>& use = faces.empty() ? last_faces : faces;
    if (use.empty()) {
        err = path + ": no faces";
        return false;
    }
    // Compact the object's vertices in first-use order (its position indices).
    std::unordered_map<long, uint32_t> remap;
    pos.clear();
    tri.clear();
    for (long g : use) {
        auto it = remap.find(g);
        if (it == remap.end()) {
            it = remap.emplace(g, (uint32_t)(pos.size() / 3)).first;
            pos.insert(pos.end(), {all[3 * g], all[3 * g + 1], all[3 * g + 2]});
        }
        tri.push_back(it->second);
    }
    return true;
}

bool build_mesh(const std::vector<float>& pos, const std::vector<uint32_t>& tri_in, MeshHost& out,
                std::string& err) {
    const size_t nv = pos.size() / 3, nt = tri_in.size() / 3;
    if (nv < 3 || nt < 1 || pos.size() % 3 || tri_in.size() % 3) {
        err = "a mesh needs at least 3 vertices and 1 triangle";
        return false;
    }
    for (uint32_t v : tri_in)
        if (v >= nv) {
            err = "triangle vertex index out of range";
            return false;
        }
    auto P = [&](uint32_t v) { return V3{pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]}; };
    // BVH over triangle centroids: median split on the longest axis, leaves of <= 4 triangles.
    std::vector<uint32_t> order(nt);
    std::iota(order.begin(), order.end(), 0u);
    std::vector<V3> cen(nt);
    for (size_t t = 0; t < nt; t++) {
        const V3 a = P(tri_in[3 * t]), b = P(tri_in[3 * t + 1]), c = P(tri_in[3 * t + 2]);
        cen[t] = mul(1.0f / 3.0f, add(add(a, b), c));
    }
    out.nodes.clear();
    out.nodes.reserve(2 * nt);
    struct Job {
        int node;
        size_t lo, hi;
    };
    out.nodes.push_back(BvhNode{});
    std::vector<Job> stack{{0, 0, nt}};
    while (!stack.empty()) {
        const Job j = stack.back();
        stack.pop_back();
        BvhNode nd{};
        for (int k = 0; k < 3; k++) {
            nd.lo[k] = INFINITY;
            nd.hi[k] = -INFINITY;
        }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = j.lo; i < j.hi; i++) {
            const uint32_t t = order[i];
            for (int c = 0; c < 3; c++) {
                const V3 p = P(tri_in[3 * t + c]);
                const float q[3] = {p.x, p.y, p.z};
                for (int k = 0; k < 3; k++) {
                    nd.lo[k] = std::min(nd.lo[k], q[k]);
                    nd.hi[k] = std::max(nd.hi[k], q[k]);
                }
            }
            const float cc[3] = {cen[t].x, cen[t].y, cen[t].z};
            for (int k = 0; k < 3; k++) {
                clo[k] = std::min(clo[k], cc[k]);
                chi[k] = std::max(chi[k], cc[k]);
            }
        }
        const size_t cnt = j.hi - j.lo;
        int axis = 0;
        for (int k = 1; k < 3; k++)
            if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
        if (cnt <= 4 || !(chi[axis] > clo[axis])) {
            nd.first = (int32_t)j.lo;
            nd.count = (int32_t)cnt;
            out.nodes[j.node] = nd;
            continue;
        }
        const size_t mid = j.lo + cnt / 2;
        auto key = [&](uint32_t t) { return axis == 0 ? cen[t].x : (axis == 1 ? cen[t].y : cen[t].z); };
        std::nth_element(order.begin() + j.lo, order.begin() + mid, order.begin() + j.hi,
                         [&](uint32_t a, uint32_t b) { return key(a) < key(b); });
        const int left = (int)out.nodes.size();
        out.nodes.push_back(BvhNode{});
        out.nodes.push_back(BvhNode{});
        nd.first = left;
        nd.count = 0;
        out.nodes[j.node] = nd;
        stack.push_back({left + 1, mid, j.hi});
        stack.push_back({left, j.lo, mid});
    }
    for (int k = 0; k < 3; k++) {
        out.lo[k] = out.nodes[0].lo[k];
        out.hi[k] = out.nodes[0].hi[k];
    }
    out.pos = pos;
    out.tri.resize(3 * nt);
    for (size_t i = 0; i < nt; i++)
        for (int c = 0; c < 3; c++) out.tri[3 * i + c] = tri_in[3 * order[i] + c];
    // Pseudonormals (MeshPseudonormals::Build): face normals; vertex normals weighted by the
    // corner angle acos(|cos|); edge normals the normalised sum of the faces sharing the edge.
    out.tri_normal.assign(3 * nt, 0.0f);
    out.edge_normal.assign(9 * nt, 0.0f);
    std::vector<V3> vn(nv, V3{0, 0, 0});
    std::unordered_map<uint64_t, V3> edges;
    auto ekey = [&](uint32_t a, uint32_t b) { return (uint64_t)std::max(a, b) + (uint64_t)std::min(a, b) * nv; };
    std::vector<V3> fn(nt);
    for (size_t t = 0; t < nt; t++) {
        const uint32_t ia = out.tri[3 * t], ib = out.tri[3 * t + 1], ic = out.tri[3 * t + 2];
        const V3 a = P(ia), b = P(ib), c = P(ic);
        const V3 cr = cross(sub(b, a), sub(c, a));
        if (!(dot(cr, cr) > 0.0f)) {
            err = "degenerate (zero-area) triangle";
            return false;
        }
        const V3 n = normalize(cr);
        fn[t] = n;
        const float a0 = std::acos(std::fabs(dot(normalize(sub(b, a)), normalize(sub(c, a)))));
        const float a1 = std::acos(std::fabs(dot(normalize(sub(a, b)), normalize(sub(c, b)))));
        const float a2 = std::acos(std::fabs(dot(normalize(sub(b, c)), normalize(sub(a, c)))));
        vn[ia] = add(vn[ia], mul(a0, n));
        vn[ib] = add(vn[ib], mul(a1, n));
        vn[ic] = add(vn[ic], mul(a2, n));
        for (auto e : {std::make_pair(ia, ib), std::make_pair(ib, ic), std::make_pair(ia, ic)}) {
            auto it = edges.find(ekey(e.first, e.second));
            if (it == edges.end())
                edges.emplace(ekey(e.first, e.second), n);
            else
                it->second = add(it->second, n);
        }
    }
    out.vertex_normal.assign(3 * nv, 0.0f);
    for (size_t v = 0; v < nv; v++) {
        if (!(dot(vn[v], vn[v]) > 0.0f)) continue;  // a vertex no triangle uses
        const V3 n = normalize(vn[v]);
        out.vertex_normal[3 * v] = n.x;
        out.vertex_normal[3 * v + 1] = n.y;
        out.vertex_normal[3 * v + 2] = n.z;
    }
    for (size_t t = 0; t < nt; t++) {
        out.tri_normal[3 * t] = fn[t].x;
        out.tri_normal[3 * t + 1] = fn[t].y;
        out.tri_normal[3 * t + 2] = fn[t].z;
        const uint32_t ia = out.tri[3 * t], ib = out.tri[3 * t + 1], ic = out.tri[3 * t + 2];
        const uint64_t ks[3] = {ekey(ia, ib), ekey(ib, ic), ekey(ia, ic)};
        for (int e = 0; e < 3; e++) {
            V3 s = edges.at(ks[e]);
            // Opposite faces of a two-sided sheet cancel: fall back to this face's normal.
            s = dot(s, s) > 0.0f ? normalize(s) : fn[t];
            out.edge_normal[9 * t + 3 * e] = s.x;
            out.edge_normal[9 * t + 3 * e + 1] = s.y;
            out.edge_normal[9 * t + 3 * e + 2] = s.z;
        }
    }
    return true;
}

}  // namespace vfs
