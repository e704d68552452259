// dg_loader.cpp -- Object::load_from_file (object.rs:106-454): an OBJ file and
// its MTL libraries turned into the arrays of Object::new.
//
// The reference reads the file with the third-party `obj` crate (kvark/obj,
// git, unpinned) and the texture images with stb_image. This file parses the
// OBJ/MTL text itself, following the published formats and the reference's use
// of the parsed data:
//   - positions, texture coordinates (u, v, 0) and normals (normalized,
//     object.rs:150-155); faces of 3 or 4 vertices, the quad split as (a, b, c)
//     and (c, d, a) (:300-371), more vertices rejected (the reference's todo!);
//   - every position scaled by 100 / (largest |v|) (:159-170);
//   - materials: [Texture::default()] followed by the MTL materials in library
//     order (:175-215), Ka/Kd/Ks required, d defaulting to 1;
//   - one mesh per non-empty group, named after it, drawn with the first
//     material of the group's name (else 0); a group with faces lacking texture
//     coordinates gets one dummy (0, 0, 0) coordinate appended (:373-388); a
//     group with faces lacking normals gets generated smooth normals over all
//     positions, accumulated from its triangles in order and normalized,
//     appended to the normals (:394-429).
// Groups follow `o`, `g` and `usemtl` the way the format defines them: `o` and
// `g` start a new group; `usemtl` sets the material in effect (which stays in
// effect for the groups that follow) and, when the current group already has
// faces, starts a new group of the same name.
// Image decoding is left to the caller (dg_obj_material returns the map paths).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/draw_gpu.h"

namespace {

struct V3f {
    float x, y, z;
};

struct Corner {
    long v, t, n;  // 0-based; -1 when absent
};

struct Group {
    std::string name, material;
    std::vector<std::vector<Corner>> faces;
};

struct Mtl {
    std::string name;
    float ka[3], kd[3], ks[3];
    bool has_ka = false, has_kd = false, has_ks = false;
    float d = 1.0f;
    std::string map_ka, map_kd;
};

}  // namespace

struct dg_obj {
    std::string name;
    std::vector<V3f> vertices, normals, uvs;
    struct Mesh {
        std::string name;
        std::vector<uint32_t> tris;  // 9 per triangle: positions, texture coordinates, normals
        int32_t texture_idx;
    };
    std::vector<Mesh> meshes;
    std::vector<Mtl> materials;  // [0] = Texture::default()
};

namespace {

std::string dir_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

bool parse_float(const std::string& s, float& out) {
    if (s.empty()) return false;
    char* end = nullptr;
    errno = 0;
    const float v = std::strtof(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') return false;
    out = v;
    return true;
}

// OBJ index: 1-based, or negative relative to the current count.
bool parse_index(const std::string& s, size_t count, long& out) {
    if (s.empty()) {
        out = -1;
        return true;
    }
    char* end = nullptr;
    const long v = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end != '\0' || v == 0) return false;
    out = v > 0 ? v - 1 : (long)count + v;
    return out >= 0;
}

std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> t;
    std::istringstream is(line);
    std::string w;
    while (is >> w) t.push_back(w);
    return t;
}

std::string rest_after(const std::string& line, const std::string& key) {
    size_t k = line.find(key);
    if (k == std::string::npos) return std::string();
    k += key.size();
    while (k < line.size() && (line[k] == ' ' || line[k] == '\t')) k++;
    size_t e = line.size();
    while (e > k && (line[e - 1] == ' ' || line[e - 1] == '\t' || line[e - 1] == '\r')) e--;
    return line.substr(k, e - k);
}

dg_status parse_mtl(const std::string& path, std::vector<Mtl>& out) {
    std::ifstream f(path);
    if (!f) return DG_E_INVALID;  // object.rs:135-137: the library must open
    std::string line;
    Mtl* cur = nullptr;
    while (std::getline(f, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        const std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        if (t[0] == "newmtl") {
            out.emplace_back();
            cur = &out.back();
            cur->name = rest_after(line, "newmtl");
            continue;
        }
        if (!cur) continue;
        auto rgb = [&](float* dst, bool& has) -> dg_status {
            if (t.size() < 4) return DG_E_INVALID;
            for (int k = 0; k < 3; k++)
                if (!parse_float(t[1 + k], dst[k])) return DG_E_INVALID;
            has = true;
            return DG_OK;
        };
        dg_status e = DG_OK;
        if (t[0] == "Ka") e = rgb(cur->ka, cur->has_ka);
        else if (t[0] == "Kd") e = rgb(cur->kd, cur->has_kd);
        else if (t[0] == "Ks") e = rgb(cur->ks, cur->has_ks);
        else if (t[0] == "d" && t.size() >= 2) e = parse_float(t[1], cur->d) ? DG_OK : DG_E_INVALID;
        else if (t[0] == "map_Ka" && t.size() >= 2) cur->map_ka = t.back();
        else if (t[0] == "map_Kd" && t.size() >= 2) cur->map_kd = t.back();
        if (e) return e;
    }
    return DG_OK;
}

void copy_str(const std::string& s, char* dst, uint64_t cap) {
    if (!dst || cap == 0) return;
    const size_t n = s.size() < cap - 1 ? s.size() : (size_t)(cap - 1);
    std::memcpy(dst, s.data(), n);
    dst[n] = '\0';
}

V3f vnormalized(V3f a) {  // linalg.rs:167-175 (norm, then three divisions)
    const float n = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return V3f{a.x / n, a.y / n, a.z / n};
}

}  // namespace

extern "C" {

dg_status dg_obj_parse(const char* path, dg_obj** out) {
    if (!path || !out) return DG_E_INVALID;
    *out = nullptr;
    std::ifstream f(path);
    if (!f) return DG_E_INVALID;  // object.rs:128: the file must open
    std::unique_ptr<dg_obj> o(new (std::nothrow) dg_obj());
    if (!o) return DG_E_OOM;
    const std::string spath(path), dir = dir_of(spath);
    o->name = spath.substr(dir.size());
    std::vector<V3f> pos, nrm, uv;
    std::vector<Group> groups(1);
    groups[0].name = "default";
    std::vector<std::string> libs;
    std::string material;  // the usemtl in effect
    std::string line;
    while (std::getline(f, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        const std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        const std::string& k = t[0];
        if (k == "v" || k == "vn") {
            V3f p;
            if (t.size() < 4 || !parse_float(t[1], p.x) || !parse_float(t[2], p.y) || !parse_float(t[3], p.z))
                return DG_E_INVALID;
            (k == "v" ? pos : nrm).push_back(p);
        } else if (k == "vt") {
            V3f p{0.0f, 0.0f, 0.0f};
            if (t.size() < 2 || !parse_float(t[1], p.x) || (t.size() >= 3 && !parse_float(t[2], p.y)))
                return DG_E_INVALID;
            uv.push_back(p);
        } else if (k == "f") {
            std::vector<Corner> face;
            for (size_t i = 1; i < t.size(); i++) {
                const std::string& c = t[i];
                const size_t s1 = c.find('/');
                const size_t s2 = s1 == std::string::npos ? std::string::npos : c.find('/', s1 + 1);
                Corner cr{-1, -1, -1};
                if (!parse_index(c.substr(0, s1), pos.size(), cr.v) || cr.v < 0) return DG_E_INVALID;
                if (s1 != std::string::npos) {
                    const std::string tt = c.substr(s1 + 1, s2 == std::string::npos ? std::string::npos : s2 - s1 - 1);
                    if (!parse_index(tt, uv.size(), cr.t)) return DG_E_INVALID;
                    if (s2 != std::string::npos && !parse_index(c.substr(s2 + 1), nrm.size(), cr.n))
                        return DG_E_INVALID;
                }
                face.push_back(cr);
            }
            groups.back().faces.push_back(std::move(face));
        } else if (k == "o" || k == "g") {
            Group g;
            g.name = t.size() >= 2 ? rest_after(line, k) : std::string("default");
            g.material = material;
            groups.push_back(std::move(g));
        } else if (k == "usemtl") {
            material = rest_after(line, "usemtl");
            if (!groups.back().faces.empty()) {
                Group g;
                g.name = groups.back().name;
                groups.push_back(std::move(g));
            }
            groups.back().material = material;
        } else if (k == "mtllib") {
            for (size_t i = 1; i < t.size(); i++) libs.push_back(t[i]);
        }
    }

    // materials: Texture::default() first (scene/mod.rs:237-252), then the libraries' (object.rs:175-215)
    Mtl def;
    def.name = "default";
    const float dka[3] = {0.9f, 0.9f, 0.9f}, dkd[3] = {0.4f, 0.4f, 0.4f}, dks[3] = {0.5f, 0.5f, 0.5f};
    std::memcpy(def.ka, dka, sizeof(dka));
    std::memcpy(def.kd, dkd, sizeof(dkd));
    std::memcpy(def.ks, dks, sizeof(dks));
    def.has_ka = def.has_kd = def.has_ks = true;
    o->materials.push_back(def);
    for (const std::string& lib : libs) {
        std::vector<Mtl> ms;
        dg_status e = parse_mtl(dir + lib, ms);
        if (e) return e;
        for (Mtl& m : ms) {
            if (!m.has_ka || !m.has_kd || !m.has_ks) return DG_E_INVALID;  // object.rs:183-185 unwrap
            if (!m.map_ka.empty()) m.map_ka = dir + m.map_ka;
            if (!m.map_kd.empty()) m.map_kd = dir + m.map_kd;
            o->materials.push_back(m);
        }
    }

    // arrays, object.rs:146-170
    for (V3f& n : nrm) n = vnormalized(n);
    if (pos.empty()) return DG_E_INVALID;  // vertices_sorted.first().unwrap()
    float vmax = -INFINITY;
    for (const V3f& p : pos) {
        const float n = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
        if (std::isnan(n)) return DG_E_INVALID;  // partial_cmp(..).unwrap() on NaN
        if (n > vmax) vmax = n;
    }
    const float factor = 100.0f / vmax;
    for (V3f& p : pos) p = V3f{p.x * factor, p.y * factor, p.z * factor};

    for (const Group& g : groups) {
        if (g.faces.empty()) continue;  // object.rs:232-235
        dg_obj::Mesh mesh;
        mesh.name = g.name;
        struct Tri {
            long v[3], t[3], n[3];
        };
        std::vector<Tri> tris;
        bool miss_t = false, miss_n = false;
        for (const std::vector<Corner>& face : g.faces) {
            if (face.size() < 3) return DG_E_INVALID;  // vertex_index[2] out of bounds
            if (face.size() > 4) return DG_E_LIMIT;    // the reference's todo!()
            bool ft = false, fn = false;
            for (const Corner& c : face) {
                if (c.v >= (long)pos.size()) return DG_E_INDEX;
                if (c.t < 0) ft = true;
                if (c.n < 0) fn = true;
                if (c.t >= (long)uv.size() || c.n >= (long)nrm.size()) return DG_E_INDEX;
            }
            miss_t |= ft;
            miss_n |= fn;
            const int orders[2][3] = {{0, 1, 2}, {2, 3, 0}};
            for (int q = 0; q < (face.size() == 4 ? 2 : 1); q++) {
                Tri tr;
                for (int k = 0; k < 3; k++) {
                    const Corner& c = face[orders[q][k]];
                    tr.v[k] = c.v;
                    tr.t[k] = ft ? -1 : c.t;
                    tr.n[k] = fn ? -1 : c.n;
                }
                tris.push_back(tr);
            }
        }
        if (miss_t) {  // one dummy texture coordinate for the group's faces without one
            const long dummy = (long)uv.size();
            uv.push_back(V3f{0.0f, 0.0f, 0.0f});
            for (Tri& tr : tris)
                if (tr.t[0] < 0) tr.t[0] = tr.t[1] = tr.t[2] = dummy;
        }
        mesh.texture_idx = 0;
        const std::string mname = g.material.empty() ? std::string("default") : g.material;
        for (size_t i = 0; i < o->materials.size(); i++)
            if (o->materials[i].name == mname) {
                mesh.texture_idx = (int32_t)i;
                break;
            }
        if (miss_n) {  // generated smooth normals over all positions, from this group's triangles
            std::vector<V3f> gen(pos.size(), V3f{0.0f, 0.0f, 0.0f});
            for (const Tri& tr : tris) {  // IndexedTriangle::calc_normal, mesh.rs:16-27: (b - a) x (c - b)
                const V3f a = pos[tr.v[0]], b = pos[tr.v[1]], c = pos[tr.v[2]];
                const V3f p{b.x - a.x, b.y - a.y, b.z - a.z}, q{c.x - b.x, c.y - b.y, c.z - b.z};
                const V3f n{(p.y * q.z) - (p.z * q.y), (p.z * q.x) - (p.x * q.z), (p.x * q.y) - (p.y * q.x)};
                for (int k = 0; k < 3; k++) {
                    V3f& s = gen[tr.v[k]];
                    s = V3f{s.x + n.x, s.y + n.y, s.z + n.z};
                }
            }
            const long base = (long)nrm.size();
            for (Tri& tr : tris)
                if (tr.n[0] < 0)
                    for (int k = 0; k < 3; k++) tr.n[k] = tr.v[k] + base;
            for (const V3f& s : gen) nrm.push_back(vnormalized(s));
        }
        for (const Tri& tr : tris) {
            for (int k = 0; k < 3; k++) mesh.tris.push_back((uint32_t)tr.v[k]);
            for (int k = 0; k < 3; k++) mesh.tris.push_back((uint32_t)tr.t[k]);
            for (int k = 0; k < 3; k++) mesh.tris.push_back((uint32_t)tr.n[k]);
        }
        o->meshes.push_back(std::move(mesh));
    }
    if (pos.size() >= 0xFFFFFFFFull || uv.size() >= 0xFFFFFFFFull || nrm.size() >= 0xFFFFFFFFull) return DG_E_LIMIT;
    o->vertices.swap(pos);
    o->normals.swap(nrm);
    o->uvs.swap(uv);
    *out = o.release();
    return DG_OK;
}

dg_status dg_obj_counts(const dg_obj* h, uint64_t* out, int32_t n) {
    if (!h || !out || n < 0) return DG_E_INVALID;
    uint64_t ntri = 0;
    for (const auto& m : h->meshes) ntri += m.tris.size() / 9;
    const uint64_t v[6] = {h->vertices.size(), h->normals.size(), h->uvs.size(), h->meshes.size(),
                           h->materials.size(), ntri};
    for (int32_t i = 0; i < n && i < 6; i++) out[i] = v[i];
    return DG_OK;
}

dg_status dg_obj_arrays(const dg_obj* h, float* vertices, float* normals, float* uvs) {
    if (!h) return DG_E_INVALID;
    if (vertices) std::memcpy(vertices, h->vertices.data(), h->vertices.size() * sizeof(V3f));
    if (normals) std::memcpy(normals, h->normals.data(), h->normals.size() * sizeof(V3f));
    if (uvs) std::memcpy(uvs, h->uvs.data(), h->uvs.size() * sizeof(V3f));
    return DG_OK;
}

dg_status dg_obj_mesh(const dg_obj* h, uint64_t mesh, uint32_t* tris, uint64_t cap, uint64_t* ntri,
                      int32_t* texture_idx, char* name, uint64_t name_cap) {
    if (!h || mesh >= h->meshes.size()) return DG_E_INVALID;
    const auto& m = h->meshes[mesh];
    if (ntri) *ntri = m.tris.size() / 9;
    if (texture_idx) *texture_idx = m.texture_idx;
    copy_str(m.name, name, name_cap);
    if (tris) {
        if (cap < m.tris.size()) return DG_E_INVALID;
        std::memcpy(tris, m.tris.data(), m.tris.size() * sizeof(uint32_t));
    }
    return DG_OK;
}

dg_status dg_obj_material(const dg_obj* h, uint64_t i, dg_material* mat, char* name, uint64_t name_cap,
                          char* map_ka, char* map_kd, uint64_t path_cap) {
    if (!h || i >= h->materials.size()) return DG_E_INVALID;
    const Mtl& m = h->materials[i];
    if (mat) {
        for (int k = 0; k < 3; k++) {
            mat->ka[k] = m.ka[k];
            mat->kd[k] = m.kd[k];
            mat->ks[k] = m.ks[k];
        }
        mat->alpha = m.d;
        mat->map_ka = -1;
        mat->map_kd = -1;
    }
    copy_str(m.name, name, name_cap);
    copy_str(m.map_ka, map_ka, path_cap);
    copy_str(m.map_kd, map_kd, path_cap);
    return DG_OK;
}

dg_status dg_obj_name(const dg_obj* h, char* name, uint64_t cap) {
    if (!h) return DG_E_INVALID;
    copy_str(h->name, name, cap);
    return DG_OK;
}

dg_status dg_obj_free(dg_obj* h) {
    if (!h) return DG_E_INVALID;
    delete h;
    return DG_OK;
}

}  // extern "C"
