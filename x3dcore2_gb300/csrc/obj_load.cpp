// Wavefront OBJ loading with the reference's rules (wavefront_obj::load_geometry,
// corelib/src/resource.cpp:137-255), without std::regex.
//
// The reference matches every line in full against four ECMAScript patterns, in this order:
//   v\s+(.+)\s+(.+)\s+(.+)\s*      vn\s+(.+)\s+(.+)\s+(.+)\s*
//   vt\s+(.+)\s+(.+)\s*            f\s+(.+)\s+(.+)\s+(.+)\s*
// where '.' is any character but '\r' (lines are split at '\n'), every quantifier is greedy and
// the groups are those of the first match in backtracking order. Lines matching none are
// ignored. Numbers are read with std::stof / std::stoul on each group (leading whitespace
// skipped, trailing text ignored, no conversion or a value out of range is an error). A face
// group splits at '/' like std::getline (a trailing empty piece is dropped) into exactly three
// pieces: vertex (required), texcoord and normal indices, 1-based and checked against the
// attributes read so far. Per vertex the mesh keeps the normal and texcoord of the last face
// corner naming it (zero when none does). The reference reads out of bounds when some face
// corner lacks a texcoord or a normal index; this loader refuses such a file instead.
//
// The matcher below is a backtracking matcher for exactly these patterns: it tries the longest
// candidate first at every quantifier, so it reports the groups std::regex reports.
#include "../../include/e8g.h"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

struct e8g_host_mesh {
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> tris;
};

namespace {

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }
bool is_any(char c) { return c != '\n' && c != '\r'; }

struct span {
    size_t b, e;
};

// PREFIX \s+ (.+) [\s+ (.+)]* \s* with `groups` groups, matched against the whole line s[0, n).
struct matcher {
    char const *s;
    size_t n;
    int groups;
    span g[3];

    // Matches "\s+ (.+)" for group k onwards from position p, then "\s*" to the end.
    bool from_ws(int k, size_t p) {
        size_t q = p;
        while (q < n && is_ws(s[q]))
            q++;
        // \s+ greedy: the longest run first, down to one character
        for (size_t w = q; w > p; w--)
            if (group(k, w))
                return true;
        return false;
    }
    bool group(int k, size_t p) {
        size_t q = p;
        while (q < n && is_any(s[q]))
            q++;
        for (size_t e = q; e > p; e--) { // (.+) greedy
            g[k] = {p, e};
            if (k + 1 < groups ? from_ws(k + 1, e) : tail(e))
                return true;
        }
        return false;
    }
    bool tail(size_t p) { // \s* to the end
        for (size_t q = p; q < n; q++)
            if (!is_ws(s[q]))
                return false;
        return true;
    }
    bool match(char const *prefix) {
        size_t l = std::strlen(prefix);
        if (n < l || std::memcmp(s, prefix, l) != 0)
            return false;
        return simple(l) || from_ws(0, l);
    }
    // The common line shape: exactly `groups` tokens after the prefix, each preceded by one space
    // or tab, no other whitespace anywhere and nothing after the last token. Then the groups are
    // the tokens (no group can take a separator, none can start with one). False when the line
    // has another shape; the backtracking matcher decides those.
    bool simple(size_t p) {
        int k = 0;
        while (p < n) {
            if (s[p] != ' ' && s[p] != '\t')
                return false;
            size_t b = ++p;
            while (p < n && !is_ws(s[p]))
                p++;
            if (p == b || k == groups)
                return false;
            g[k++] = {b, p};
        }
        return k == groups;
    }
};

// A group as its own NUL-terminated string (the reference converts the matched substring alone).
struct group_text {
    char small[96];
    std::string big;
    char const *c_str;
    group_text(char const *s, span g) {
        size_t len = g.e - g.b;
        if (len < sizeof(small)) {
            std::memcpy(small, s + g.b, len);
            small[len] = 0;
            c_str = small;
        } else {
            big.assign(s + g.b, len);
            c_str = big.c_str();
        }
    }
};

struct obj_error {
    std::string msg;
};

// std::stof: strtof over the string, an error when nothing converts or the value is out of range.
float to_float(char const *b) {
    char *end = nullptr;
    int saved = errno;
    errno = 0;
    float v = std::strtof(b, &end);
    bool range = errno == ERANGE;
    if (errno == 0)
        errno = saved;
    if (end == b)
        throw obj_error{std::string("stof: no conversion of \"") + b + "\""};
    if (range)
        throw obj_error{std::string("stof: \"") + b + "\" out of range"};
    return v;
}

// std::stoul (base 10, unsigned long) cast to unsigned, as the reference casts it.
uint32_t to_index(char const *b) {
    char *end = nullptr;
    int saved = errno;
    errno = 0;
    unsigned long v = std::strtoul(b, &end, 10);
    bool range = errno == ERANGE;
    if (errno == 0)
        errno = saved;
    if (end == b)
        throw obj_error{std::string("stoul: no conversion of \"") + b + "\""};
    if (range)
        throw obj_error{std::string("stoul: \"") + b + "\" out of range"};
    return static_cast<uint32_t>(v);
}

// std::getline-style split of s[g.b, g.e) at '/': empty pieces kept, except a trailing one.
// Returns the number of pieces; the first three are stored in p.
int split_slash(char const *s, span g, span p[3]) {
    int n = 0;
    size_t b = g.b;
    while (b < g.e) {
        size_t e = b;
        while (e < g.e && s[e] != '/')
            e++;
        if (n < 3)
            p[n] = {b, e};
        n++;
        if (e == g.e)
            break;
        b = e + 1;
    }
    return n;
}

void parse(char const *text, size_t len, e8g_host_mesh &out) {
    std::vector<float> verts, norms, tex;
    std::vector<uint32_t> iv, in, it;
    verts.reserve(len / 24);
    iv.reserve(len / 16);
    size_t line_no = 0, b = 0;
    auto at = [&line_no]() { return " at line " + std::to_string(line_no); };
    while (b < len) {
        size_t e = b;
        while (e < len && text[e] != '\n')
            e++;
        matcher m{text + b, e - b, 3, {}};
        b = e + 1;
        line_no++;
        if (m.n == 0)
            continue;
        char c0 = m.s[0];
        if (c0 != 'v' && c0 != 'f')
            continue; // matches none of the four patterns
        if (m.match("v")) {
            for (int k = 0; k < 3; k++)
                verts.push_back(to_float(group_text(m.s, m.g[k]).c_str));
        } else if (m.match("vn")) {
            for (int k = 0; k < 3; k++)
                norms.push_back(to_float(group_text(m.s, m.g[k]).c_str));
        } else if ((m.groups = 2, m.match("vt"))) {
            tex.push_back(to_float(group_text(m.s, m.g[0]).c_str));
            tex.push_back(to_float(group_text(m.s, m.g[1]).c_str));
        } else if ((m.groups = 3, m.match("f"))) {
            for (int k = 0; k < 3; k++) {
                span p[3];
                if (split_slash(m.s, m.g[k], p) != 3)
                    throw obj_error{"malformed face" + at() + ": a corner needs vertex/texcoord/normal"};
                if (p[0].e == p[0].b)
                    throw obj_error{"malformed face" + at() + ": vertex index missing"};
                uint32_t v = to_index(group_text(m.s, p[0]).c_str) - 1;
                if (v >= verts.size() / 3)
                    throw obj_error{"face" + at() + " references an undefined vertex"};
                iv.push_back(v);
                if (p[1].e != p[1].b) {
                    uint32_t t = to_index(group_text(m.s, p[1]).c_str) - 1;
                    if (t >= tex.size() / 2)
                        throw obj_error{"face" + at() + " references an undefined texcoord"};
                    it.push_back(t);
                }
                if (p[2].e != p[2].b) {
                    uint32_t n = to_index(group_text(m.s, p[2]).c_str) - 1;
                    if (n >= norms.size() / 3)
                        throw obj_error{"face" + at() + " references an undefined normal"};
                    in.push_back(n);
                }
            }
        }
    }
    if (verts.empty())
        throw obj_error{"the mesh has no vertex data"};
    if (it.size() != iv.size() || in.size() != iv.size())
        throw obj_error{"every face corner needs texcoord and normal indices"};
    size_t nv = verts.size() / 3, nf = iv.size() / 3;
    out.pos = std::move(verts);
    out.nrm.assign(3 * nv, 0.0f);
    out.uv.assign(2 * nv, 0.0f);
    for (size_t c = 0; c < 3 * nf; c++) {
        for (int k = 0; k < 3; k++)
            out.nrm[3 * static_cast<size_t>(iv[c]) + k] = norms[3 * static_cast<size_t>(in[c]) + k];
        for (int k = 0; k < 2; k++)
            out.uv[2 * static_cast<size_t>(iv[c]) + k] = tex[2 * static_cast<size_t>(it[c]) + k];
    }
    out.tris = std::move(iv);
}

void set_err(char *err, size_t err_len, std::string const &msg) {
    if (err && err_len) {
        std::snprintf(err, err_len, "%s", msg.c_str());
    }
}

} // namespace

extern "C" {

e8g_status e8g_obj_parse(char const *text, size_t len, e8g_host_mesh **out, char *err, size_t err_len) {
    if (!out || (!text && len))
        return E8G_ERR_INVALID_ARG;
    *out = nullptr;
    e8g_host_mesh *m = nullptr;
    try {
        m = new e8g_host_mesh();
        parse(text, len, *m);
    } catch (obj_error const &x) {
        delete m;
        set_err(err, err_len, x.msg);
        return E8G_ERR_INVALID_ARG;
    } catch (std::bad_alloc const &) {
        delete m;
        set_err(err, err_len, "out of host memory");
        return E8G_ERR_OUT_OF_MEMORY;
    }
    *out = m;
    return E8G_OK;
}

e8g_status e8g_obj_load(char const *path, e8g_host_mesh **out, char *err, size_t err_len) {
    if (!path || !out)
        return E8G_ERR_INVALID_ARG;
    *out = nullptr;
    std::string text;
    try {
        std::ifstream f(path, std::ios::binary);
        if (!f.is_open()) {
            set_err(err, err_len, std::string("cannot open ") + path);
            return E8G_ERR_INVALID_ARG;
        }
        std::ostringstream ss;
        ss << f.rdbuf();
        text = ss.str();
    } catch (std::bad_alloc const &) {
        set_err(err, err_len, "out of host memory");
        return E8G_ERR_OUT_OF_MEMORY;
    }
    return e8g_obj_parse(text.data(), text.size(), out, err, err_len);
}

e8g_status e8g_host_mesh_data(e8g_host_mesh const *m, e8g_mesh_data *d) {
    if (!m || !d)
        return E8G_ERR_INVALID_ARG;
    d->num_vertices = static_cast<uint32_t>(m->pos.size() / 3);
    d->num_triangles = static_cast<uint32_t>(m->tris.size() / 3);
    d->positions = m->pos.data();
    d->normals = m->nrm.data();
    d->texcoords = m->uv.data();
    d->triangles = m->tris.data();
    return E8G_OK;
}

void e8g_host_mesh_free(e8g_host_mesh *m) { delete m; }

} // extern "C"
