// Synthetic scene generators. Every random quantity comes from SplitMix64 streams keyed by the
// generator seed, so a (kind, seed, sizes) triple names one scene on every host.
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <unordered_map>

namespace {

uint64_t splitmix64(uint64_t &state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct rng64 {
    uint64_t s;
    explicit rng64(uint64_t seed) : s(seed) {}
    double uniform() { return static_cast<double>(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    uint32_t below(uint32_t n) { return static_cast<uint32_t>(uniform() * n) % n; }
};

struct vec3d {
    double x, y, z;
};
vec3d operator+(vec3d a, vec3d b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
vec3d operator-(vec3d a, vec3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
vec3d operator*(vec3d a, double k) { return {a.x * k, a.y * k, a.z * k}; }
double dot(vec3d a, vec3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
vec3d cross(vec3d a, vec3d b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
vec3d normalize(vec3d a) {
    double l = std::sqrt(dot(a, a));
    return l > 0 ? a * (1.0 / l) : a;
}

e8g_material lambert(float r, float g, float b) {
    e8g_material m{};
    m.type = E8G_MAT_OREN_NAYAR;
    m.albedo[0] = r;
    m.albedo[1] = g;
    m.albedo[2] = b;
    m.roughness = 0.0f;
    m.mix0 = m.mix1 = -1;
    return m;
}

e8g_material metal(float r, float g, float b, float roughness, float f0) {
    e8g_material m{};
    m.type = E8G_MAT_COOK_TORR;
    m.albedo[0] = r;
    m.albedo[1] = g;
    m.albedo[2] = b;
    m.roughness = roughness;
    float s = std::sqrt(f0);
    m.ior_re = (1.0f + s) / (1.0f - s); // Schlick F0 as a real index of refraction
    m.ior_im = 0.0f;
    m.mix0 = m.mix1 = -1;
    return m;
}

// Camera looking from eye to target; rot columns are (right, up, back) as pinhole_camera's
// direction = R * (x, y, -f) expects.
e8g_camera look_at(vec3d eye, vec3d target, vec3d up, float vfov_deg, float aspect) {
    vec3d f = normalize(target - eye);
    vec3d r = normalize(cross(f, up));
    vec3d u = cross(r, f);
    e8g_camera c{};
    c.origin[0] = static_cast<float>(eye.x);
    c.origin[1] = static_cast<float>(eye.y);
    c.origin[2] = static_cast<float>(eye.z);
    double cols[3][3] = {{r.x, r.y, r.z}, {u.x, u.y, u.z}, {-f.x, -f.y, -f.z}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            c.rot[3 * i + j] = static_cast<float>(cols[j][i]);
    c.focal_len = 1.0f;
    c.sensor_size = static_cast<float>(2.0 * std::tan(vfov_deg * 0.5 * M_PI / 180.0));
    c.aspect = aspect;
    return c;
}

void push3(std::vector<float> &v, vec3d p) {
    v.push_back(static_cast<float>(p.x));
    v.push_back(static_cast<float>(p.y));
    v.push_back(static_cast<float>(p.z));
}

// A planar quad a-b-c-d as two triangles with a flat normal n.
void add_quad(e8g_host_scene *s, vec3d a, vec3d b, vec3d c, vec3d d, vec3d n, int32_t mat) {
    std::vector<float> p, nn;
    push3(p, a);
    push3(p, b);
    push3(p, c);
    push3(p, d);
    for (int i = 0; i < 4; i++)
        push3(nn, n);
    s->add_mesh(p, nn, {0, 1, 2, 0, 2, 3}, mat);
}

// Closed box of half extents h, rotated by angle (radians) about +y, centred at c.
void add_box(e8g_host_scene *s, vec3d c, vec3d h, double angle, int32_t mat) {
    double ca = std::cos(angle), sa = std::sin(angle);
    auto xf = [&](vec3d p) {
        return vec3d{c.x + ca * p.x + sa * p.z, c.y + p.y, c.z - sa * p.x + ca * p.z};
    };
    auto xn = [&](vec3d n) { return vec3d{ca * n.x + sa * n.z, n.y, -sa * n.x + ca * n.z}; };
    std::vector<float> p, nn;
    std::vector<uint32_t> t;
    const vec3d normals[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int f = 0; f < 6; f++) {
        vec3d n = normals[f];
        vec3d a = std::fabs(n.y) > 0.5 ? vec3d{1, 0, 0} : vec3d{0, 1, 0};
        vec3d b = cross(n, a);
        vec3d corners[4] = {n + a * -1 + b * -1, n + a + b * -1, n + a + b, n + a * -1 + b};
        uint32_t base = static_cast<uint32_t>(p.size() / 3);
        for (auto q : corners) {
            push3(p, xf({q.x * h.x, q.y * h.y, q.z * h.z}));
            push3(nn, xn(n));
        }
        t.insert(t.end(), {base, base + 1, base + 2, base, base + 2, base + 3});
    }
    s->add_mesh(p, nn, t, mat);
}

double lattice(uint64_t seed, int64_t x, int64_t y, int64_t z) {
    uint64_t st = seed ^ (static_cast<uint64_t>(x) * 0x9E3779B1ull) ^
                  (static_cast<uint64_t>(y) * 0x85EBCA77ull << 1) ^
                  (static_cast<uint64_t>(z) * 0xC2B2AE3Dull << 2);
    splitmix64(st);
    return static_cast<double>(splitmix64(st) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

double value_noise(uint64_t seed, vec3d p) {
    double fx = std::floor(p.x), fy = std::floor(p.y), fz = std::floor(p.z);
    int64_t ix = static_cast<int64_t>(fx), iy = static_cast<int64_t>(fy), iz = static_cast<int64_t>(fz);
    double tx = p.x - fx, ty = p.y - fy, tz = p.z - fz;
    auto fade = [](double t) { return t * t * (3 - 2 * t); };
    tx = fade(tx);
    ty = fade(ty);
    tz = fade(tz);
    double v = 0;
    for (int dz = 0; dz < 2; dz++)
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                double w = (dx ? tx : 1 - tx) * (dy ? ty : 1 - ty) * (dz ? tz : 1 - tz);
                v += w * lattice(seed, ix + dx, iy + dy, iz + dz);
            }
    return v;
}

// Three octaves (frequency x2, amplitude /2), normalised to [-1, 1].
double noise3(uint64_t seed, vec3d p) {
    double v = 0, amp = 1, norm = 0, freq = 4.0;
    for (int o = 0; o < 3; o++) {
        v += amp * value_noise(seed + 0x1000u * o, p * freq);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return v / norm;
}

// Icosphere of the given level: 20 * 4^level faces.
void icosphere(unsigned level, std::vector<vec3d> &verts, std::vector<uint32_t> &faces) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    verts = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
             {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto &v : verts)
        v = normalize(v);
    faces = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
             3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (unsigned l = 0; l < level; l++) {
        std::unordered_map<uint64_t, uint32_t> mid;
        mid.reserve(faces.size() * 2);
        std::vector<uint32_t> nf;
        nf.reserve(faces.size() * 4);
        auto midpoint = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? (static_cast<uint64_t>(a) << 32 | b) : (static_cast<uint64_t>(b) << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end())
                return it->second;
            verts.push_back(normalize((verts[a] + verts[b]) * 0.5));
            uint32_t id = static_cast<uint32_t>(verts.size() - 1);
            mid.emplace(key, id);
            return id;
        };
        for (size_t f = 0; f < faces.size(); f += 3) {
            uint32_t a = faces[f], b = faces[f + 1], c = faces[f + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            nf.insert(nf.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
        }
        faces.swap(nf);
    }
}

// Splits a triangle set with per-face material ids into one mesh per material (a corelib
// trimesh carries a single material), keeping the shared smooth normals.
void add_by_material(e8g_host_scene *s, std::vector<vec3d> const &v, std::vector<vec3d> const &n,
                     std::vector<uint32_t> const &faces, std::vector<uint32_t> const &face_mat,
                     uint32_t num_mats, int32_t mat_base) {
    std::vector<std::vector<uint32_t>> by(num_mats);
    for (size_t f = 0; f < face_mat.size(); f++)
        by[face_mat[f]].push_back(static_cast<uint32_t>(f));
    std::vector<uint32_t> remap(v.size(), 0xFFFFFFFFu);
    for (uint32_t m = 0; m < num_mats; m++) {
        if (by[m].empty())
            continue;
        std::vector<float> p, nn;
        std::vector<uint32_t> t;
        std::vector<uint32_t> used;
        for (uint32_t f : by[m]) {
            for (int k = 0; k < 3; k++) {
                uint32_t g = faces[3 * f + k];
                if (remap[g] == 0xFFFFFFFFu) {
                    remap[g] = static_cast<uint32_t>(p.size() / 3);
                    push3(p, v[g]);
                    push3(nn, n[g]);
                    used.push_back(g);
                }
                t.push_back(remap[g]);
            }
        }
        for (uint32_t g : used)
            remap[g] = 0xFFFFFFFFu;
        s->add_mesh(p, nn, t, mat_base + static_cast<int32_t>(m));
    }
}

} // namespace

namespace e8g_gen {

// Cornell box: unit-cube room (floor, ceiling, back, red left, green right walls as Lambert
// quads), two boxes rotated about y, a 0.25 x 0.25 ceiling light of radiance (17, 12, 4) made of
// two equal-area triangles; 40 degree vertical field of view. 36 triangles.
e8g_host_scene *cornell(e8g_gen_opts const &o) {
    auto s = new e8g_host_scene();
    s->mats = {lambert(0.73f, 0.73f, 0.73f), lambert(0.63f, 0.065f, 0.05f), lambert(0.14f, 0.45f, 0.09f),
               lambert(0.0f, 0.0f, 0.0f)};
    add_quad(s, {0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, 0);  // floor
    add_quad(s, {0, 1, 0}, {0, 1, 1}, {1, 1, 1}, {1, 1, 0}, {0, -1, 0}, 0); // ceiling
    add_quad(s, {0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 1}, 0);  // back
    add_quad(s, {0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0}, 1);  // left, red
    add_quad(s, {1, 0, 0}, {1, 1, 0}, {1, 1, 1}, {1, 0, 1}, {-1, 0, 0}, 2); // right, green
    add_box(s, {0.66, 0.15, 0.62}, {0.15, 0.15, 0.15}, -18.0 * M_PI / 180.0, 0);
    add_box(s, {0.34, 0.30, 0.36}, {0.15, 0.30, 0.15}, 15.0 * M_PI / 180.0, 0);
    uint32_t lm = static_cast<uint32_t>(s->mesh_mat.size());
    add_quad(s, {0.375, 0.999, 0.375}, {0.375, 0.999, 0.625}, {0.625, 0.999, 0.625},
             {0.625, 0.999, 0.375}, {0, -1, 0}, 3);
    s->lights.push_back(e8g_light{lm, {17.0f, 12.0f, 4.0f}});
    float aspect = o.height ? static_cast<float>(o.width) / static_cast<float>(o.height) : 1.0f;
    // 3% margin around the opening so no primary ray grazes its edges exactly
    double d = 0.515 / std::tan(20.0 * M_PI / 180.0);
    s->cam = look_at({0.5, 0.5, 1.0 + d}, {0.5, 0.5, 0.0}, {0, 1, 0}, 40.0f, aspect);
    return s;
}

// Icosphere of the given level displaced along its normals by seeded 3-octave value noise,
// over a 2-triangle ground plane, lit by 4 quad lights; num_materials materials with albedo
// U[0.1,0.9]^3 and roughness U[rough_lo, rough_hi], odd ones metallic (cook_torr, F0 U[0.5,1)),
// even ones Lambert; one material per face, uniform.
e8g_host_scene *displaced_icosphere(e8g_gen_opts const &o) {
    auto s = new e8g_host_scene();
    rng64 rng(o.seed * 0x2545F4914F6CDD1Dull + 17);
    uint32_t nm = o.num_materials ? o.num_materials : 512;
    float rlo = o.roughness_hi > 0 ? o.roughness_lo : 0.05f;
    float rhi = o.roughness_hi > 0 ? o.roughness_hi : 0.8f;
    for (uint32_t m = 0; m < nm; m++) {
        float a0 = static_cast<float>(rng.uniform(0.1, 0.9));
        float a1 = static_cast<float>(rng.uniform(0.1, 0.9));
        float a2 = static_cast<float>(rng.uniform(0.1, 0.9));
        float r = static_cast<float>(rng.uniform(rlo, rhi));
        float f0 = static_cast<float>(rng.uniform(0.5, 0.98));
        if (m & 1)
            s->mats.push_back(metal(a0, a1, a2, r, f0));
        else {
            e8g_material l = lambert(a0, a1, a2);
            l.roughness = 0.0f;
            s->mats.push_back(l);
        }
    }
    int32_t ground_mat = static_cast<int32_t>(s->mats.size());
    s->mats.push_back(lambert(0.6f, 0.6f, 0.6f));
    int32_t light_mat = static_cast<int32_t>(s->mats.size());
    s->mats.push_back(lambert(0.0f, 0.0f, 0.0f));

    std::vector<vec3d> v;
    std::vector<uint32_t> f;
    icosphere(o.level, v, f);
    const double R = 0.5;
    const vec3d C{0.0, 0.62, 0.0};
    float amp = o.amplitude > 0 ? o.amplitude : 0.05f;
    uint64_t nseed = o.seed * 0x9E3779B97F4A7C15ull + 3;
    for (auto &p : v) {
        double d = R + amp * noise3(nseed, p);
        p = C + p * d;
    }
    std::vector<vec3d> n(v.size(), vec3d{0, 0, 0});
    for (size_t i = 0; i < f.size(); i += 3) {
        vec3d a = v[f[i]], b = v[f[i + 1]], c = v[f[i + 2]];
        vec3d fn = cross(b - a, c - a); // area weighted, outward for this winding
        n[f[i]] = n[f[i]] + fn;
        n[f[i + 1]] = n[f[i + 1]] + fn;
        n[f[i + 2]] = n[f[i + 2]] + fn;
    }
    for (size_t i = 0; i < n.size(); i++) {
        n[i] = normalize(n[i]);
        if (dot(n[i], v[i] - C) < 0)
            n[i] = n[i] * -1.0;
    }
    std::vector<uint32_t> fm(f.size() / 3);
    for (auto &x : fm)
        x = rng.below(nm);
    add_by_material(s, v, n, f, fm, nm, 0);

    add_quad(s, {-3, 0, -3}, {-3, 0, 3}, {3, 0, 3}, {3, 0, -3}, {0, 1, 0}, ground_mat);
    const double ly = 2.2, hs = 0.3;
    const vec3d lc[4] = {{-1.2, ly, -1.0}, {1.2, ly, -1.0}, {-1.0, ly, 1.3}, {1.0, ly, 1.3}};
    const float lr[4][3] = {{9.0f, 8.0f, 7.0f}, {7.0f, 8.0f, 9.0f}, {8.0f, 8.0f, 8.0f}, {10.0f, 9.0f, 6.0f}};
    for (int l = 0; l < 4; l++) {
        vec3d c = lc[l];
        uint32_t lm = static_cast<uint32_t>(s->mesh_mat.size());
        add_quad(s, {c.x - hs, c.y, c.z - hs}, {c.x + hs, c.y, c.z - hs}, {c.x + hs, c.y, c.z + hs},
                 {c.x - hs, c.y, c.z + hs}, {0, -1, 0}, light_mat);
        s->lights.push_back(e8g_light{lm, {lr[l][0], lr[l][1], lr[l][2]}});
    }
    float aspect = o.height ? static_cast<float>(o.width) / static_cast<float>(o.height) : 16.0f / 9.0f;
    s->cam = look_at({0.0, 1.0, 2.1}, {0.0, 0.55, 0.0}, {0, 1, 0}, 40.0f, aspect);
    return s;
}

// Seeded random triangle soup of num_tris triangles inside [-1, 1]^3, enclosed by a room box
// with an area light under its ceiling; 8 materials with roughness U[rough_lo, rough_hi].
e8g_host_scene *soup(e8g_gen_opts const &o) {
    auto s = new e8g_host_scene();
    rng64 rng(o.seed * 0xD1B54A32D192ED03ull + 99);
    const uint32_t nm = 8;
    float rlo = o.roughness_hi > 0 ? o.roughness_lo : 0.02f;
    float rhi = o.roughness_hi > 0 ? o.roughness_hi : 1.0f;
    for (uint32_t m = 0; m < nm; m++) {
        float a0 = static_cast<float>(rng.uniform(0.2, 0.9));
        float a1 = static_cast<float>(rng.uniform(0.2, 0.9));
        float a2 = static_cast<float>(rng.uniform(0.2, 0.9));
        float r = static_cast<float>(rng.uniform(rlo, rhi));
        if (m & 1)
            s->mats.push_back(metal(a0, a1, a2, r, static_cast<float>(rng.uniform(0.5, 0.95))));
        else
            s->mats.push_back(lambert(a0, a1, a2));
    }
    int32_t room_mat = static_cast<int32_t>(s->mats.size());
    s->mats.push_back(lambert(0.7f, 0.7f, 0.7f));
    int32_t light_mat = static_cast<int32_t>(s->mats.size());
    s->mats.push_back(lambert(0.0f, 0.0f, 0.0f));

    uint32_t nt = o.num_tris ? o.num_tris : 1000;
    double size = 2.0 / std::cbrt(static_cast<double>(nt)) * 1.2;
    std::vector<vec3d> v;
    std::vector<vec3d> n;
    std::vector<uint32_t> f, fm;
    for (uint32_t t = 0; t < nt; t++) {
        vec3d c{rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)};
        vec3d p[3];
        for (int k = 0; k < 3; k++)
            p[k] = c + vec3d{rng.uniform(-size, size), rng.uniform(-size, size), rng.uniform(-size, size)};
        vec3d fn = normalize(cross(p[1] - p[0], p[2] - p[0]));
        for (int k = 0; k < 3; k++) {
            v.push_back(p[k]);
            n.push_back(fn);
            f.push_back(static_cast<uint32_t>(v.size() - 1));
        }
        fm.push_back(rng.below(nm));
    }
    add_by_material(s, v, n, f, fm, nm, 0);
    const double B = 1.6;
    add_quad(s, {-B, -B, -B}, {B, -B, -B}, {B, -B, B}, {-B, -B, B}, {0, 1, 0}, room_mat);
    add_quad(s, {-B, B, -B}, {-B, B, B}, {B, B, B}, {B, B, -B}, {0, -1, 0}, room_mat);
    add_quad(s, {-B, -B, -B}, {-B, B, -B}, {B, B, -B}, {B, -B, -B}, {0, 0, 1}, room_mat);
    add_quad(s, {-B, -B, B}, {B, -B, B}, {B, B, B}, {-B, B, B}, {0, 0, -1}, room_mat);
    add_quad(s, {-B, -B, -B}, {-B, -B, B}, {-B, B, B}, {-B, B, -B}, {1, 0, 0}, room_mat);
    add_quad(s, {B, -B, -B}, {B, B, -B}, {B, B, B}, {B, -B, B}, {-1, 0, 0}, room_mat);
    uint32_t lm = static_cast<uint32_t>(s->mesh_mat.size());
    const double L = 0.5, ly = B - 1e-3;
    add_quad(s, {-L, ly, -L}, {-L, ly, L}, {L, ly, L}, {L, ly, -L}, {0, -1, 0}, light_mat);
    s->lights.push_back(e8g_light{lm, {12.0f, 11.0f, 10.0f}});
    float aspect = o.height ? static_cast<float>(o.width) / static_cast<float>(o.height) : 1.0f;
    s->cam = look_at({0.0, 0.0, B - 0.05}, {0.0, 0.0, 0.0}, {0, 1, 0}, 60.0f, aspect);
    return s;
}

// The reference's furnace scene (tst_pathtracer.cpp:24-56): uv_sphere(o = 0, r = 10, res,
// flip_normal = true) built with the same float arithmetic as uv_sphere's constructor
// (geometry.cpp:162-241), Lambert (oren_nayar sigma 0) albedo 0.7, area light L = 1 on the same
// mesh; camera at the centre. The analytic sum of RGB radiance is 3 * 1 / (1 - 0.7) = 10.
e8g_host_scene *furnace(e8g_gen_opts const &o) {
    auto s = new e8g_host_scene();
    unsigned res = o.level ? o.level : 30;
    float r = 10.0f;
    std::vector<float> p, n;
    std::vector<uint32_t> t;
    auto pushf = [](std::vector<float> &a, float x, float y, float z) {
        a.push_back(x);
        a.push_back(y);
        a.push_back(z);
    };
    pushf(p, 0.0f, 0.0f, -r);
    pushf(n, 0.0f, 0.0f, 1.0f);
    for (unsigned j = 1; j < res - 1; j++) {
        float u = static_cast<float>(j) / res;
        float phi = (1 - u) * static_cast<float>(M_PI);
        for (unsigned i = 0; i < res; i++) {
            float vv = static_cast<float>(i) / res;
            float theta = vv * static_cast<float>(2 * M_PI);
            float x = std::sin(phi) * std::cos(theta);
            float y = std::sin(phi) * std::sin(theta);
            float z = std::cos(phi);
            pushf(p, r * x + 0.0f, r * y + 0.0f, r * z + 0.0f);
            pushf(n, -1.0f * x, -1.0f * y, -1.0f * z);
        }
    }
    pushf(p, 0.0f, 0.0f, r);
    pushf(n, 0.0f, 0.0f, -1.0f);
    for (unsigned i = 1; i < res + 1; i++)
        t.insert(t.end(), {i % res + 1, i, 0u});
    for (unsigned j = 1; j < res - 2; j++)
        for (unsigned i = 1; i < res + 1; i++) {
            t.insert(t.end(), {i % res + 1 + j * res, i + j * res, i + (j - 1) * res});
            t.insert(t.end(), {i % res + 1 + (j - 1) * res, i % res + 1 + j * res, i + (j - 1) * res});
        }
    for (unsigned i = 1; i < res + 1; i++)
        t.insert(t.end(), {i % res + 1 + (res - 3) * res, 1 + (res - 2) * res, i + (res - 3) * res});
    s->mats.push_back(lambert(0.7f, 0.7f, 0.7f));
    uint32_t m = s->add_mesh(p, n, t, 0);
    s->lights.push_back(e8g_light{m, {1.0f, 1.0f, 1.0f}});
    s->cam = e8g_camera{};
    s->cam.rot[0] = s->cam.rot[4] = s->cam.rot[8] = 1.0f;
    s->cam.focal_len = 1.0f;
    s->cam.sensor_size = static_cast<float>(2.0 * std::tan(20.0 * M_PI / 180.0));
    s->cam.aspect = 1.0f;
    return s;
}

} // namespace e8g_gen

char const *e8g_validate_desc(e8g_scene_desc const *d) {
    if (!d)
        return "scene description is NULL";
    if (d->num_meshes == 0)
        return "scene has no meshes";
    if (!d->mesh_vert_offset || !d->mesh_tri_offset || !d->positions || !d->normals || !d->triangles)
        return "scene arrays are NULL";
    if (d->mesh_vert_offset[0] != 0 || d->mesh_tri_offset[0] != 0)
        return "mesh offsets must start at 0";
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        if (d->mesh_vert_offset[m + 1] < d->mesh_vert_offset[m] || d->mesh_tri_offset[m + 1] < d->mesh_tri_offset[m])
            return "mesh offsets must not decrease";
        uint32_t nv = d->mesh_vert_offset[m + 1] - d->mesh_vert_offset[m];
        for (uint32_t t = d->mesh_tri_offset[m]; t < d->mesh_tri_offset[m + 1]; t++)
            for (int k = 0; k < 3; k++)
                if (d->triangles[3 * t + k] >= nv)
                    return "triangle index out of range of its mesh";
        if (d->mesh_material && d->mesh_material[m] >= static_cast<int32_t>(d->num_materials))
            return "mesh material index out of range";
    }
    uint32_t nv_total = d->mesh_vert_offset[d->num_meshes];
    for (size_t i = 0; i < 3 * static_cast<size_t>(nv_total); i++)
        if (!std::isfinite(d->positions[i]) || !std::isfinite(d->normals[i]))
            return "vertex positions and normals must be finite";
    e8g_camera const &cam = d->camera;
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(cam.origin[k]))
            return "camera origin must be finite";
    for (int k = 0; k < 9; k++)
        if (!std::isfinite(cam.rot[k]))
            return "camera rotation must be finite";
    if (!(cam.sensor_size > 0) || !(cam.focal_len > 0) || !(cam.aspect > 0) || !std::isfinite(cam.sensor_size) ||
        !std::isfinite(cam.focal_len) || !std::isfinite(cam.aspect))
        return "camera sensor size, focal length and aspect must be finite and positive";
    if (d->num_lights == 0)
        return "scene has no lights";
    for (uint32_t l = 0; l < d->num_lights; l++) {
        if (d->lights[l].mesh >= d->num_meshes)
            return "light mesh index out of range";
        if (d->mesh_tri_offset[d->lights[l].mesh + 1] == d->mesh_tri_offset[d->lights[l].mesh])
            return "light mesh has no triangles";
        for (int k = 0; k < 3; k++)
            if (!std::isfinite(d->lights[l].radiance[k]) || d->lights[l].radiance[k] < 0)
                return "light radiance must be finite and non-negative";
    }
    // the light CDF divides by the total power (lightsources.cpp:45-52): some light must emit
    double total = 0;
    for (uint32_t l = 0; l < d->num_lights; l++) {
        e8g_light const &L = d->lights[l];
        uint32_t m = L.mesh, v0 = d->mesh_vert_offset[m];
        double area = 0;
        for (uint32_t t = d->mesh_tri_offset[m]; t < d->mesh_tri_offset[m + 1]; t++) {
            float const *a = d->positions + 3 * static_cast<size_t>(v0 + d->triangles[3 * t]);
            float const *b = d->positions + 3 * static_cast<size_t>(v0 + d->triangles[3 * t + 1]);
            float const *c = d->positions + 3 * static_cast<size_t>(v0 + d->triangles[3 * t + 2]);
            double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            double x = u[1] * w[2] - u[2] * w[1], y = u[2] * w[0] - u[0] * w[2], z = u[0] * w[1] - u[1] * w[0];
            area += 0.5 * std::sqrt(x * x + y * y + z * z);
        }
        total += area * (L.radiance[0] + L.radiance[1] + L.radiance[2]);
    }
    if (!(total > 0))
        return "the lights emit no power (zero radiance or zero area)";
    for (uint32_t i = 0; i < d->num_materials; i++) {
        e8g_material const &m = d->materials[i];
        if (m.type > E8G_MAT_MIXTURE)
            return "unknown material type";
        if (!std::isfinite(m.albedo[0]) || !std::isfinite(m.albedo[1]) || !std::isfinite(m.albedo[2]) ||
            !std::isfinite(m.roughness) || !std::isfinite(m.ior_re) || !std::isfinite(m.ior_im) ||
            !std::isfinite(m.ratio))
            return "material values must be finite";
        if (m.type == E8G_MAT_MIXTURE) {
            if (m.mix0 < 0 || m.mix1 < 0 || m.mix0 >= static_cast<int32_t>(d->num_materials) ||
                m.mix1 >= static_cast<int32_t>(d->num_materials))
                return "mixture component index out of range";
            if (d->materials[m.mix0].type == E8G_MAT_MIXTURE || d->materials[m.mix1].type == E8G_MAT_MIXTURE)
                return "mixture components must not be mixtures";
        }
    }
    return nullptr;
}

extern "C" {

e8g_status e8g_scene_validate(e8g_scene_desc const *d, char *msg, size_t cap) {
    char const *bad = e8g_validate_desc(d);
    if (msg && cap) {
        std::snprintf(msg, cap, "%s", bad ? bad : "");
    }
    return bad ? E8G_ERR_INVALID_ARG : E8G_OK;
}

e8g_status e8g_gen_scene(e8g_gen_opts const *o, e8g_host_scene **out) {
    if (!o || !out)
        return E8G_ERR_INVALID_ARG;
    try {
        switch (o->kind) {
        case E8G_GEN_CORNELL:
            *out = e8g_gen::cornell(*o);
            break;
        case E8G_GEN_DISPLACED_ICO:
            if (o->level > 10)
                return E8G_ERR_INVALID_ARG;
            *out = e8g_gen::displaced_icosphere(*o);
            break;
        case E8G_GEN_SOUP:
            *out = e8g_gen::soup(*o);
            break;
        case E8G_GEN_FURNACE:
            if (o->level != 0 && o->level < 4)
                return E8G_ERR_INVALID_ARG;
            *out = e8g_gen::furnace(*o);
            break;
        default:
            return E8G_ERR_INVALID_ARG;
        }
    } catch (...) {
        return E8G_ERR_OUT_OF_MEMORY;
    }
    return E8G_OK;
}

e8g_status e8g_host_scene_desc(e8g_host_scene const *s, e8g_scene_desc *desc) {
    if (!s || !desc)
        return E8G_ERR_INVALID_ARG;
    *desc = s->desc();
    return E8G_OK;
}

void e8g_host_scene_free(e8g_host_scene *s) { delete s; }

} // extern "C"
