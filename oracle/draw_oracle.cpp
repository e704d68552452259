// draw_oracle.cpp -- CPU restatement of the draw renderer (TEST INFRASTRUCTURE, see draw_oracle.h).
//
// Every function below names the reference code it restates (paths relative
// to the mororo18/draw project). Floating-point expressions keep the Rust
// evaluation order: left-associative, no contraction, IEEE f32 division and
// square root, Rust's saturating float->int casts, wrapping usize/u8 arithmetic
// where the reference runs in release mode.
#include "draw_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

namespace {

// ----------------------------------------------------------------- linalg.rs
const float EPS = 0.0000001f;  // linalg.rs:6

struct Vec2 {
    float x, y;
};
inline Vec2 operator+(Vec2 a, Vec2 b) { return {a.x + b.x, a.y + b.y}; }        // linalg.rs:29-35
inline Vec2 operator-(Vec2 a, Vec2 b) { return a + Vec2{-b.x, -b.y}; }           // linalg.rs:37-43
inline Vec2 operator*(Vec2 a, float s) { return {a.x * s, a.y * s}; }            // linalg.rs:45-54
inline Vec2 operator/(Vec2 a, float s) { return {a.x / s, a.y / s}; }            // linalg.rs:56-65

struct Vec3 {
    float a[3];
    float x() const { return a[0]; }
    float y() const { return a[1]; }
    float z() const { return a[2]; }
    // linalg.rs:167-171: powi(2) is x*x; the sum is left-associative.
    float norm() const {
        float sum = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        return std::sqrt(sum);
    }
    Vec3 normalized() const;                                                      // linalg.rs:173-175
    float dot(const Vec3& b) const { return a[0] * b.a[0] + a[1] * b.a[1] + a[2] * b.a[2]; }  // :182-184
    Vec3 cross(const Vec3& b) const {                                             // linalg.rs:186-200
        float c0 = (a[1] * b.a[2]) - (a[2] * b.a[1]);
        float c1 = (a[2] * b.a[0]) - (a[0] * b.a[2]);
        float c2 = (a[0] * b.a[1]) - (a[1] * b.a[0]);
        return Vec3{{c0, c1, c2}};
    }
};
inline Vec3 V3(float x, float y, float z) { return Vec3{{x, y, z}}; }
inline Vec3 operator*(Vec3 v, float s) { return V3(v.a[0] * s, v.a[1] * s, v.a[2] * s); }   // :213-221
inline Vec3 operator/(Vec3 v, float s) { return V3(v.a[0] / s, v.a[1] / s, v.a[2] / s); }   // :223-231
inline Vec3 operator+(Vec3 u, Vec3 v) { return V3(u.a[0] + v.a[0], u.a[1] + v.a[1], u.a[2] + v.a[2]); }
inline Vec3 operator-(Vec3 u, Vec3 v) { return V3(u.a[0] - v.a[0], u.a[1] - v.a[1], u.a[2] - v.a[2]); }
Vec3 Vec3::normalized() const { return *this / norm(); }
inline Vec3 color_multiply(Vec3 u, Vec3 v) { return V3(u.x() * v.x(), u.y() * v.y(), u.z() * v.z()); }  // canvas.rs:13-17

struct Vec4 {
    float a[4];
};
inline Vec4 as_vec4(Vec3 v) { return Vec4{{v.a[0], v.a[1], v.a[2], 1.0f}}; }    // linalg.rs:163-165

struct Matrix4 {
    float a[4][4];
    static Matrix4 zeros() {
        Matrix4 m;
        std::memset(&m, 0, sizeof(m));
        return m;
    }
    Matrix4 transposed() const {                                                  // linalg.rs:275-287
        Matrix4 c = *this;
        for (int i = 0; i < 4; i++)
            for (int j = i + 1; j < 4; j++) {
                float t = c.a[i][j];
                c.a[i][j] = c.a[j][i];
                c.a[j][i] = t;
            }
        return c;
    }
    static Matrix4 rotate_y(float theta) {                                        // linalg.rs:301-311
        float s = std::sin(theta), co = std::cos(theta);
        Matrix4 m = zeros();
        m.a[0][0] = co; m.a[0][2] = s;
        m.a[1][1] = 1.0f;
        m.a[2][0] = -s; m.a[2][2] = co;
        m.a[3][3] = 1.0f;
        return m;
    }
};
// linalg.rs:328-344 and :346-360: accumulators start at 0.0 and add k = 0..3 in order.
inline Matrix4 operator*(const Matrix4& x, const Matrix4& y) {
    Matrix4 c = Matrix4::zeros();
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++) c.a[i][j] += x.a[i][k] * y.a[k][j];
    return c;
}
inline Vec4 operator*(const Matrix4& m, const Vec4& v) {
    Vec4 o{{0.0f, 0.0f, 0.0f, 0.0f}};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) o.a[i] += m.a[i][j] * v.a[j];
    return o;
}
inline Vec3 vec3_over_w(const Vec4& v) { return V3(v.a[0], v.a[1], v.a[2]) / v.a[3]; }   // linalg.rs:89-91

// Rust `as usize` / `as u8` on f32: saturating, NaN -> 0.
inline uint64_t as_usize(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}
inline uint8_t as_u8(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 255.0f) return 255;
    return (uint8_t)(unsigned)f;
}

// ----------------------------------------------------------------- canvas.rs
struct Pixel {  // canvas.rs:51-59, memory order b,g,r,padd
    uint8_t b, g, r, padd;
};
inline Pixel pixel_new(uint8_t r, uint8_t g, uint8_t b) { return Pixel{b, g, r, 255}; }   // :63-70
inline Vec3 normalized_as_vec3(Pixel p) {                                                 // :81-87
    return V3((float)p.r / 255.0f, (float)p.g / 255.0f, (float)p.b / 255.0f);
}
inline Pixel from_normalized_vec3(Vec3 s) {                                               // :89-92
    Vec3 sc = s * 255.0f;
    return pixel_new(as_u8(sc.x()), as_u8(sc.y()), as_u8(sc.z()));
}
inline Pixel pixel_add(Pixel a, Pixel b) {  // :136-152, release-mode wrapping u8 add, padd = 0
    return Pixel{(uint8_t)(a.b + b.b), (uint8_t)(a.g + b.g), (uint8_t)(a.r + b.r), 0};
}
inline Pixel pixel_mul(Pixel a, float s) {  // :154-169
    return Pixel{as_u8((float)a.b * s), as_u8((float)a.g * s), as_u8((float)a.r * s), 0};
}
inline Pixel azul_bb() { return pixel_new(155, 186, 255); }  // :131-133

const int MAXL = OR_MAX_LIGHTS;

// VertexAttributes (canvas.rs:193-291) extended with one light/halfway pair per light.
struct Attr {
    Vec3 normal;
    Vec3 light[MAXL];
    Vec3 halfway[MAXL];
    Vec3 texture_coord;
    Vec2 screen_coord;
    float depth;
};
// The Add/Sub/Mul impls (canvas.rs:242-291) act field by field.
Attr attr_add(const Attr& p, const Attr& q, int nl) {
    Attr r;
    r.screen_coord = p.screen_coord + q.screen_coord;
    r.depth = p.depth + q.depth;
    r.normal = p.normal + q.normal;
    for (int l = 0; l < nl; l++) r.light[l] = p.light[l] + q.light[l];
    for (int l = 0; l < nl; l++) r.halfway[l] = p.halfway[l] + q.halfway[l];
    r.texture_coord = p.texture_coord + q.texture_coord;
    return r;
}
Attr attr_sub(const Attr& p, const Attr& q, int nl) {
    Attr r;
    r.screen_coord = p.screen_coord - q.screen_coord;
    r.depth = p.depth - q.depth;
    r.normal = p.normal - q.normal;
    for (int l = 0; l < nl; l++) r.light[l] = p.light[l] - q.light[l];
    for (int l = 0; l < nl; l++) r.halfway[l] = p.halfway[l] - q.halfway[l];
    r.texture_coord = p.texture_coord - q.texture_coord;
    return r;
}
Attr attr_mul(const Attr& p, float t, int nl) {
    Attr r;
    r.screen_coord = p.screen_coord * t;
    r.depth = p.depth * t;
    r.normal = p.normal * t;
    for (int l = 0; l < nl; l++) r.light[l] = p.light[l] * t;
    for (int l = 0; l < nl; l++) r.halfway[l] = p.halfway[l] * t;
    r.texture_coord = p.texture_coord * t;
    return r;
}

struct Rect {  // canvas.rs:293-351 (usize arithmetic)
    uint64_t x, y, w, h;
    uint64_t x_min() const { return x; }
    uint64_t y_min() const { return y; }
    uint64_t x_max() const { return x + w; }
    uint64_t y_max() const { return y + h; }
    static Rect from_coords(uint64_t x0, uint64_t y0, uint64_t x1, uint64_t y1) {
        uint64_t xmn = std::min(x0, x1), ymn = std::min(y0, y1);
        uint64_t xmx = std::max(x0, x1), ymx = std::max(y0, y1);
        return Rect{xmn, ymn, xmx - xmn, ymx - ymn};
    }
    static Rect clip(const Rect& a, const Rect& b) {
        uint64_t x_min = std::max(a.x, b.x), y_min = std::max(a.y, b.y);
        uint64_t x_max = std::min(a.x + a.w, b.x + b.w), y_max = std::min(a.y + a.h, b.y + b.h);
        if (x_min > x_max) { x_min = 0; x_max = 0; }
        if (y_min > y_max) { y_min = 0; y_max = 0; }
        return from_coords(x_min, y_min, x_max, y_max);
    }
};

// ----------------------------------------------------- scene/mod.rs textures
struct TextureMap {  // scene/mod.rs:102-126
    std::vector<uint8_t> img;
    uint64_t width = 0, height = 0, components = 0;
    float f_width = 0, f_height = 0;
    int filter = OR_FILTER_NEAREST;  // extension: OR_FILTER_BILINEAR (no counterpart in the reference)
};
std::shared_ptr<TextureMap> texmap_default() {  // scene/mod.rs:128-135 (white, 1x1, 3 comps)
    auto t = std::make_shared<TextureMap>();
    t->img = {255, 255, 255};
    t->width = t->height = 1;
    t->components = 3;
    t->f_width = 1.0f;
    t->f_height = 1.0f;
    return t;
}
// get_rgb_slice, scene/mod.rs:154-168. usize math wraps (release); the slice
// index panics when offset+3 exceeds the image, reported as OR_E_TEXTURE_RANGE.
bool get_rgb_slice(const TextureMap& t, float u, float v, uint8_t out[3]) {
    uint64_t u_idx = as_usize(std::floor(u * (t.f_width - 1.0f)));
    uint64_t v_idx = t.height - 1 - as_usize(std::floor(v * (t.f_height - 1.0f)));
    uint64_t off = (v_idx * t.width + u_idx) * t.components;
    uint64_t len = t.img.size();
    if (len < 3 || off > len - 3) return false;
    out[0] = t.img[off];
    out[1] = t.img[off + 1];
    out[2] = t.img[off + 2];
    return true;
}
// Extension (no counterpart in the reference, which samples the nearest texel
// above): bilinear fetch. x = u * (W - 1) and y = v * (H - 1) as in
// get_rgb_slice; the base texel (x0, y0) = (floor x, floor y) is addressed
// exactly like the nearest texel (same wrapping offset); its neighbours are
// x0 + 1 (when x0 + 1 < W, else x0 again) and y0 + 1 (the row above in memory,
// when that row exists, else y0 again). Every texel's three bytes become
// byte / 255; per channel, with ax = x - x0 and ay = y - y0:
//   t0 = c(x0, y0) * (1 - ax) + c(x0 + 1, y0) * ax
//   t1 = c(x0, y0 + 1) * (1 - ax) + c(x0 + 1, y0 + 1) * ax
//   c  = t0 * (1 - ay) + t1 * ay
// evaluated left to right in f32 without contraction. Any of the four offsets
// past the image is the texture-range error, like the reference's slice index.
bool get_rgb_bilinear(const TextureMap& t, float u, float v, Vec3& out) {
    const float x = u * (t.f_width - 1.0f), y = v * (t.f_height - 1.0f);
    const float fx = std::floor(x), fy = std::floor(y);
    const float ax = x - fx, ay = y - fy;
    const uint64_t u_idx = as_usize(fx);
    const uint64_t v_idx = t.height - 1 - as_usize(fy);
    const uint64_t off00 = (v_idx * t.width + u_idx) * t.components;
    const uint64_t dx = (u_idx + 1 < t.width) ? t.components : 0;
    const uint64_t dy = (v_idx >= 1 && v_idx < t.height) ? t.width * t.components : 0;
    const uint64_t off[4] = {off00, off00 + dx, off00 - dy, off00 - dy + dx};
    const uint64_t len = t.img.size();
    for (int k = 0; k < 4; k++)
        if (len < 3 || off[k] > len - 3) return false;
    float ch[3];
    for (int i = 0; i < 3; i++) {
        const float c00 = (float)t.img[off[0] + i] / 255.0f, c01 = (float)t.img[off[1] + i] / 255.0f;
        const float c10 = (float)t.img[off[2] + i] / 255.0f, c11 = (float)t.img[off[3] + i] / 255.0f;
        const float t0 = c00 * (1.0f - ax) + c01 * ax;
        const float t1 = c10 * (1.0f - ax) + c11 * ax;
        ch[i] = t0 * (1.0f - ay) + t1 * ay;
    }
    out = V3(ch[0], ch[1], ch[2]);
    return true;
}
// The diffuse/ambient sample of a map under its filter mode (nearest: the
// reference's get_rgb_slice and Pixel::normalized_as_vec3).
bool sample_rgb(const TextureMap& t, float u, float v, Vec3& out);

// get_rgba_slice, scene/mod.rs:137-152.
bool get_rgba_slice(const TextureMap& t, float u, float v, uint8_t out[4]) {
    uint64_t u_idx = as_usize(std::floor(u * t.f_width));
    uint64_t v_idx = t.height - 1 - as_usize(std::floor(v * t.f_height));
    uint64_t off = (v_idx * t.width + u_idx) * t.components;
    uint64_t len = t.img.size();
    if (len < 4 || off > len - 4) return false;
    for (int i = 0; i < 4; i++) out[i] = t.img[off + i];
    return true;
}

struct Texture {  // scene/mod.rs:206-216
    Vec3 ka, kd, ks;
    float alpha;
    std::shared_ptr<TextureMap> map_ka, map_kd;
};
Texture texture_default() {  // scene/mod.rs:237-252
    return Texture{V3(0.9f, 0.9f, 0.9f), V3(0.4f, 0.4f, 0.4f), V3(0.5f, 0.5f, 0.5f), 1.0f, texmap_default(),
                   texmap_default()};
}

bool sample_rgb(const TextureMap& t, float u, float v, Vec3& out) {
    if (t.filter == OR_FILTER_BILINEAR) return get_rgb_bilinear(t, u, v, out);
    uint8_t s[3];
    if (!get_rgb_slice(t, u, v, s)) return false;
    out = normalized_as_vec3(pixel_new(s[0], s[1], s[2]));
    return true;
}

// -------------------------------------------------------------- Canvas state
struct Canvas {
    std::vector<Pixel> frame;
    uint64_t width = 0, height = 0;
    Vec2 offset{0.0f, 0.0f};
    bool depth_update_enabled = false;
    std::vector<float> depth_frame;
    float depth_max = 0.0f;
    int err = OR_OK;

    void init_depth(float d) {  // canvas.rs:403-411
        depth_max = d;
        if (depth_frame.size() != frame.size())
            depth_frame.assign(frame.size(), d);
        else
            std::fill(depth_frame.begin(), depth_frame.end(), d);
    }
    void clear() {  // canvas.rs:425-433
        std::fill(frame.begin(), frame.end(), azul_bb());
        if (!depth_frame.empty()) init_depth(depth_max);
    }
    Vec2 pos_map_center(Vec2 p) const { return Vec2{std::floor(p.x + 0.5f), std::floor(p.y + 0.5f)}; }  // :896-904
    Pixel get_pixel_coord(uint64_t x, uint64_t y) const { return frame[width * (height - y - 1) + x]; }  // :932-944
    void draw_pixel_coord(uint64_t x, uint64_t y, Pixel c) { frame[width * (height - y - 1) + x] = c; }  // :946-960
    // canvas.rs:906-930
    void draw_pixel_coord_with_depth(uint64_t x, uint64_t y, Pixel color, float opacity, float depth) {
        Pixel nc = color;
        if (opacity < 1.0f) {
            Pixel bg = get_pixel_coord(x, y);
            nc = pixel_add(pixel_mul(bg, 1.0f - opacity), pixel_mul(color, opacity));
        }
        if (depth < depth_frame[width * y + x]) {
            draw_pixel_coord(x, y, nc);
            if (depth_update_enabled) depth_frame[width * y + x] = depth;
        }
    }
};

// Edge functions of canvas.rs:597-616 (f_ab, f_bc, f_ca share one shape).
inline float edge(Vec2 p, Vec2 q, float x, float y) {
    return (p.y - q.y) * x + (q.x - p.x) * y + (p.x * q.y) - (q.x * p.y);
}
inline float min3(float a, float b, float c) {  // canvas.rs:618-627 (NaN-skipping)
    float r = INFINITY;
    for (float v : {a, b, c})
        if (v < r) r = v;
    return r;
}
inline float max3(float a, float b, float c) {  // canvas.rs:629-638
    float r = -INFINITY;
    for (float v : {a, b, c})
        if (v > r) r = v;
    return r;
}

inline float powi(float a, int b) {  // LLVM powi lowering: binary exponentiation from r = 1
    bool recip = b < 0;
    unsigned n = recip ? 0u - (unsigned)b : (unsigned)b;
    float r = 1.0f;
    while (true) {
        if (n & 1u) r = r * a;
        n >>= 1;
        if (n == 0) break;
        a = a * a;
    }
    return recip ? 1.0f / r : r;
}

// Canvas::draw_triangle_with_attributes, canvas.rs:577-750 (clipping_rect = None).
// w holds the three vertices' clip-space w (the projection's fourth row); it is
// used only by the perspective-correct extension (interp ==
// OR_INTERP_PERSPECTIVE, no counterpart in the reference): with the reference's
// screen-space barycentrics alpha, beta, gama,
//   pa = alpha * (1 / w_a), pb = beta * (1 / w_b), pc = gama * (1 / w_c)
//   s = (pa + pb) + pc,  qa = pa / s, qb = pb / s, qc = pc / s
// and texture coordinates, normals, light and halfway vectors are interpolated
// as (a * qa + b * qb) + c * qc. Coverage and depth (the interpolated eye
// distance) keep the reference's screen-space barycentrics in both modes.
void draw_triangle_with_attributes(Canvas& cv, const Attr& A, const Attr& B, const Attr& C, const Texture& tex,
                                   int nl, int exponent, const float w[3], int interp) {
    Vec2 a = cv.pos_map_center(A.screen_coord - cv.offset);
    Vec2 b = cv.pos_map_center(B.screen_coord - cv.offset);
    Vec2 c = cv.pos_map_center(C.screen_coord - cv.offset);
    float a_depth = A.depth, b_depth = B.depth, c_depth = C.depth;

    uint64_t x_min = as_usize(min3(a.x, b.x, c.x));
    uint64_t y_min = as_usize(min3(a.y, b.y, c.y));
    uint64_t x_max = as_usize(max3(a.x, b.x, c.x));
    uint64_t y_max = as_usize(max3(a.y, b.y, c.y));
    Rect drawable = Rect::from_coords(x_min, y_min, x_max, y_max);
    Rect screen = Rect::from_coords(0, 0, cv.width - 1, cv.height - 1);
    drawable = Rect::clip(drawable, screen);
    Rect valid = Rect::clip(screen, drawable);
    x_min = valid.x_min();
    y_min = valid.y_min();
    x_max = valid.x_max();
    y_max = valid.y_max();

    float f_alpha = edge(b, c, a.x, a.y);
    float f_beta = edge(c, a, b.x, b.y);
    float f_gama = edge(a, b, c.x, c.y);
    float f_alpha_out = edge(b, c, -1.0f, -1.0f);
    float f_beta_out = edge(c, a, -1.0f, -1.0f);
    float f_gama_out = edge(a, b, -1.0f, -1.0f);

    for (uint64_t y = y_min; y <= y_max; y++) {
        float yf = (float)y;
        for (uint64_t x = x_min; x <= x_max; x++) {
            float xf = (float)x;
            float alpha = edge(b, c, xf, yf) / f_alpha;
            float beta = edge(c, a, xf, yf) / f_beta;
            float gama = edge(a, b, xf, yf) / f_gama;
            if (!(alpha >= 0.0f && beta >= 0.0f && gama >= 0.0f)) continue;
            if (!((alpha > 0.0f || f_alpha * f_alpha_out > 0.0f) && (beta > 0.0f || f_beta * f_beta_out > 0.0f) &&
                  (gama > 0.0f || f_gama * f_gama_out > 0.0f)))
                continue;
            float pixel_depth = (alpha * a_depth) + (beta * b_depth) + (gama * c_depth);
            if (interp == OR_INTERP_PERSPECTIVE) {
                const float pa = alpha * (1.0f / w[0]), pb = beta * (1.0f / w[1]), pc = gama * (1.0f / w[2]);
                const float sw = (pa + pb) + pc;
                alpha = pa / sw;
                beta = pb / sw;
                gama = pc / sw;
            }
            Vec3 ptc = (A.texture_coord * alpha) + (B.texture_coord * beta) + (C.texture_coord * gama);
            Vec3 diffuse, ambient;
            if (!sample_rgb(*tex.map_kd, ptc.x(), ptc.y(), diffuse) ||
                !sample_rgb(*tex.map_ka, ptc.x(), ptc.y(), ambient)) {
                cv.err = OR_E_TEXTURE_RANGE;
                return;
            }
            Vec3 pn = (A.normal * alpha) + (B.normal * beta) + (C.normal * gama);
            Vec3 c_l = tex.ks;
            Vec3 c_r = color_multiply(diffuse, tex.kd);
            Vec3 c_a = color_multiply(ambient, tex.ka);
            // canvas.rs:736-739 with one light; further lights add their terms in order.
            Vec3 inner = c_a;
            Vec3 spec;
            for (int l = 0; l < nl; l++) {
                Vec3 pl = (A.light[l] * alpha) + (B.light[l] * beta) + (C.light[l] * gama);
                float ln = pl.dot(pn);
                float mx = (ln > 0.0f) ? ln : 0.0f;  // 0.0_f32.max(ln): NaN -> 0
                inner = inner + c_l * (1.0f - mx);
            }
            Vec3 col = color_multiply(c_r, inner);
            for (int l = 0; l < nl; l++) {
                Vec3 ph = (A.halfway[l] * alpha) + (B.halfway[l] * beta) + (C.halfway[l] * gama);
                spec = c_l * powi(ph.dot(pn), exponent);
                col = col + spec;
            }
            Pixel color = from_normalized_vec3(col);
            cv.draw_pixel_coord_with_depth(x, y, color, tex.alpha, pixel_depth);
        }
    }
}

// ------------------------------------------------------- scene/mod.rs camera
struct ViewPlane {  // scene/mod.rs:596-660
    Vec3 normal;
    float k;
    float func(const Vec3& p) const { return normal.dot(p) + k; }
};

struct Camera {  // scene/mod.rs:282-594
    Vec3 position, direction, up;
    float top, bottom, right, left;
    float min_view_dist, max_view_dist;
    Vec3 u, v, w;
};

int camera_new(Camera& cam, Vec3 pos, Vec3 dir, float ratio, float near_, float far_, float fov_x) {
    const float RADS_PER_DEG = 3.14159265358979323846f / 180.0f;  // f32::to_radians
    float fov_x_rad = fov_x * RADS_PER_DEG;
    float right = std::fabs(near_) * std::tan(fov_x_rad / 2.0f);
    float left = -right;
    float top = (1.0f / ratio) * right;
    float bottom = -top;
    if (!(fov_x < 180.0f) || !(near_ < 0.0f) || !(near_ > far_) || !(right > left) || !(top > bottom))
        return OR_E_CAMERA;
    cam.position = pos;
    cam.direction = dir.normalized();
    cam.up = V3(0.0f, 1.0f, 0.0f);
    cam.top = top;
    cam.bottom = bottom;
    cam.right = right;
    cam.left = left;
    cam.min_view_dist = near_;
    cam.max_view_dist = far_;
    cam.u = cam.v = cam.w = V3(0, 0, 0);
    return OR_OK;
}

void update_basis(Camera& c) {  // scene/mod.rs:438-451
    Vec3 g = c.direction;
    Vec3 w = (g / g.norm()) * (-1.0f);
    Vec3 t_x_w = c.up.cross(w);
    Vec3 u = t_x_w / t_x_w.norm();
    Vec3 v = w.cross(u);
    c.u = u.normalized();
    c.v = v.normalized();
    c.w = w.normalized();
}

int basis_matrix(const Camera& c, Matrix4& m) {  // scene/mod.rs:415-428
    if (!(c.u.norm() > 0.0f && c.v.norm() > 0.0f && c.w.norm() > 0.0f)) return OR_E_CAMERA;
    m = Matrix4::zeros();
    m.a[0][0] = c.u.x(); m.a[0][1] = c.v.x(); m.a[0][2] = c.w.x();
    m.a[1][0] = c.u.y(); m.a[1][1] = c.v.y(); m.a[1][2] = c.w.y();
    m.a[2][0] = c.u.z(); m.a[2][1] = c.v.z(); m.a[2][2] = c.w.z();
    m.a[3][3] = 1.0f;
    return OR_OK;
}

int gen_matrix(Camera& c, Matrix4& out) {  // scene/mod.rs:453-479
    Vec3 p = c.position;
    Matrix4 mp = Matrix4::zeros();
    mp.a[0][0] = 1.0f; mp.a[0][3] = -p.x();
    mp.a[1][1] = 1.0f; mp.a[1][3] = -p.y();
    mp.a[2][2] = 1.0f; mp.a[2][3] = -p.z();
    mp.a[3][3] = 1.0f;
    update_basis(c);
    Matrix4 b;
    int e = basis_matrix(c, b);
    if (e) return e;
    out = b.transposed() * mp;
    return OR_OK;
}

int plane_new(const Vec3 pts[3], Vec3 visible, ViewPlane& pl) {  // scene/mod.rs:603-632
    Vec3 p = pts[1] - pts[0];
    Vec3 q = pts[2] - pts[1];
    Vec3 n = p.cross(q);
    float k = -n.dot(pts[0]);
    float t = n.dot(visible) + k;
    if (t < 0.0f) {
        n = q.cross(p);
        k = -n.dot(pts[0]);
        t = n.dot(visible) + k;
        if (!(t > 0.0f)) return OR_E_CAMERA;
    }
    pl.normal = n;
    pl.k = k;
    return OR_OK;
}

// gen_view_planes, scene/mod.rs:481-593: planes[0]=near, [1]=far, [2..6]=right,left,top,bottom.
int gen_view_planes(Camera& c, ViewPlane planes[6]) {
    update_basis(c);
    Matrix4 mb;
    int e = basis_matrix(c, mb);
    if (e) return e;
    Vec3 cp = c.position;
    float n = c.min_view_dist, f = c.max_view_dist;
    float r = c.right, l = c.left, t = c.top, b = c.bottom;
    auto world = [&](Vec3 v) { return vec3_over_w(mb * as_vec4(v)) + cp; };
    Vec3 urn = world(V3(r, t, n));
    Vec3 uln = world(V3(l, t, n));
    Vec3 lrn = world(V3(r, b, n));
    Vec3 lln = world(V3(l, b, n));
    float xc = (l + r) / 2.0f;
    float yc = (b + t) / 2.0f;
    Vec3 ucf = world(V3(xc, (f * t) / n, f));
    Vec3 lcf = world(V3(xc, (f * b) / n, f));
    Vec3 rcf = world(V3((f * r) / n, yc, f));
    Vec3 lfc = world(V3((f * l) / n, yc, f));
    Vec3 vis = (urn + lcf) / 2.0f;
    Vec3 p0[3] = {urn, lrn, lln};
    Vec3 p1[3] = {lfc, rcf, ucf};
    Vec3 p2[3] = {rcf, urn, lrn};
    Vec3 p3[3] = {lfc, lln, uln};
    Vec3 p4[3] = {ucf, uln, urn};
    Vec3 p5[3] = {lcf, lln, lrn};
    const Vec3* all[6] = {p0, p1, p2, p3, p4, p5};
    for (int i = 0; i < 6; i++) {
        e = plane_new(all[i], vis, planes[i]);
        if (e) return e;
    }
    return OR_OK;
}

// ------------------------------------------------ scene/mod.rs triangles/clip
struct Triangle {
    Vec3 v[3];
    Attr at[3];
};
Vec3 calc_normal(const Triangle& t) { return (t.v[1] - t.v[0]).cross(t.v[2] - t.v[1]); }  // :30-41
Vec3 get_center(const Triangle& t) {                                                     // :92-99
    Vec3 s = V3(0, 0, 0);
    for (int i = 0; i < 3; i++) s = s + t.v[i];
    return s / 3.0f;
}
bool at_least_partially_visible(const ViewPlane& p, const Triangle& t) {  // :641-660
    float fa = p.func(t.v[0]), fb = p.func(t.v[1]), fc = p.func(t.v[2]);
    if (fa > 0.0f && fb > 0.0f && fc > 0.0f) return true;
    if (fa <= 0.0f && fb <= 0.0f && fc <= 0.0f) return false;
    return true;
}
// ViewPlane::clip, scene/mod.rs:662-746.
int plane_clip(const ViewPlane& p, const Triangle& t, Triangle* out, int nl) {
    Vec3 a = t.v[0], b = t.v[1], c = t.v[2];
    Attr aa = t.at[0], ba = t.at[1], ca = t.at[2];
    float fa = p.func(a), fb = p.func(b), fc = p.func(c);
    if (fa > 0.0f && fb > 0.0f && fc > 0.0f) {
        out[0] = t;
        return 1;
    } else if (fa <= 0.0f && fb <= 0.0f && fc <= 0.0f) {
        return 0;
    }
    if (fa * fc >= 0.0f) {
        std::swap(fb, fc); std::swap(b, c); std::swap(ba, ca);
        std::swap(fa, fb); std::swap(a, b); std::swap(aa, ba);
    } else if (fb * fc >= 0.0f) {
        std::swap(fa, fc); std::swap(a, c); std::swap(aa, ca);
        std::swap(fa, fb); std::swap(a, b); std::swap(aa, ba);
    }
    float t_a = p.func(a) / p.normal.dot(a - c) - EPS;
    Vec3 na = a + (c - a) * t_a;
    Attr naa = attr_add(aa, attr_mul(attr_sub(ca, aa, nl), t_a, nl), nl);
    float t_b = p.func(b) / p.normal.dot(b - c) - EPS;
    Vec3 nb = b + (c - b) * t_b;
    Attr nba = attr_add(ba, attr_mul(attr_sub(ca, ba, nl), t_b, nl), nl);
    if (fc <= 0.0f) {
        out[0].v[0] = a; out[0].v[1] = na; out[0].v[2] = nb;
        out[0].at[0] = aa; out[0].at[1] = naa; out[0].at[2] = nba;
        out[1].v[0] = a; out[1].v[1] = b; out[1].v[2] = nb;
        out[1].at[0] = aa; out[1].at[1] = ba; out[1].at[2] = nba;
        return 2;
    }
    out[0].v[0] = c; out[0].v[1] = na; out[0].v[2] = nb;
    out[0].at[0] = ca; out[0].at[1] = naa; out[0].at[2] = nba;
    return 1;
}
// Triangle::clip_against_planes, scene/mod.rs:43-90.
int clip_against_planes(const Triangle& t, const ViewPlane planes[6], Triangle* ret, int nl) {
    int n = 0;
    if (at_least_partially_visible(planes[2], t) && at_least_partially_visible(planes[3], t) &&
        at_least_partially_visible(planes[4], t) && at_least_partially_visible(planes[5], t)) {
        ret[0] = t;
        n = 1;
    }
    Triangle tmp[12];
    Triangle* cur = ret;
    Triangle* nxt = tmp;
    for (int d = 0; d < 2; d++) {
        int nn = 0;
        for (int i = 0; i < n; i++) nn += plane_clip(planes[d], cur[i], nxt + nn, nl);
        std::swap(cur, nxt);
        n = nn;
    }
    if (cur != ret)
        for (int i = 0; i < n; i++) ret[i] = cur[i];
    return n;
}

// ------------------------------------------------------------ objects, scene
struct Mesh {  // mesh.rs:30-35
    std::vector<uint32_t> tris;  // 9 per triangle: pos[3], uv[3], nrm[3]
    int32_t texture_idx;
};
struct Object {  // object.rs:18-31
    std::vector<Vec3> vertices, normals, uvs;
    std::vector<Mesh> opaque, transparent;
    std::vector<Texture> textures;
};
struct Scene {  // scene/mod.rs:749-757
    uint64_t width, height;
    Camera camera;
    std::vector<int32_t> objects;
    std::vector<Vec3> lights;
    int exponent = 2;
    int interpolation = OR_INTERP_AFFINE;  // extension: OR_INTERP_PERSPECTIVE
};

}  // namespace

struct or_ctx {
    std::vector<std::shared_ptr<TextureMap>> texmaps;
    std::vector<std::shared_ptr<Object>> objects;
    std::vector<Scene> scenes;
    std::vector<Canvas> canvases;
};

extern "C" {

or_ctx* or_ctx_new(void) { return new or_ctx(); }
void or_ctx_free(or_ctx* c) { delete c; }

int32_t or_texmap_new(or_ctx* c, const uint8_t* img, uint64_t len, uint64_t w, uint64_t h, uint64_t comps) {
    if (comps == 0 || len % comps != 0 || len / comps != w * h) return -OR_E_INVALID;  // scene/mod.rs:114-115
    auto t = std::make_shared<TextureMap>();
    t->img.assign(img, img + len);
    t->width = w;
    t->height = h;
    t->components = comps;
    t->f_width = (float)w;
    t->f_height = (float)h;
    c->texmaps.push_back(t);
    return (int32_t)c->texmaps.size() - 1;
}

int32_t or_object_new(or_ctx* c, const float* vertices, uint64_t nv, const float* normals, uint64_t nn,
                      const float* uvs, uint64_t nuv, const uint32_t* tris, const uint64_t* mesh_ntri,
                      const int32_t* mesh_tex, uint64_t nmesh, const or_material* mats, uint64_t nmat) {
    auto o = std::make_shared<Object>();
    for (uint64_t i = 0; i < nv; i++) o->vertices.push_back(V3(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]));
    for (uint64_t i = 0; i < nn; i++) o->normals.push_back(V3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]));
    for (uint64_t i = 0; i < nuv; i++) o->uvs.push_back(V3(uvs[3 * i], uvs[3 * i + 1], uvs[3 * i + 2]));
    for (uint64_t i = 0; i < nmat; i++) {
        Texture t;
        t.ka = V3(mats[i].ka[0], mats[i].ka[1], mats[i].ka[2]);
        t.kd = V3(mats[i].kd[0], mats[i].kd[1], mats[i].kd[2]);
        t.ks = V3(mats[i].ks[0], mats[i].ks[1], mats[i].ks[2]);
        t.alpha = mats[i].alpha;
        for (int k = 0; k < 2; k++) {
            int32_t id = k == 0 ? mats[i].map_ka : mats[i].map_kd;
            std::shared_ptr<TextureMap> m;
            if (id < 0)
                m = texmap_default();
            else if ((size_t)id < c->texmaps.size())
                m = c->texmaps[id];
            else
                return -OR_E_INVALID;
            (k == 0 ? t.map_ka : t.map_kd) = m;
        }
        o->textures.push_back(t);
    }
    uint64_t off = 0;
    for (uint64_t m = 0; m < nmesh; m++) {
        Mesh mesh;
        mesh.texture_idx = mesh_tex[m];
        // object.rs:46-48: textures[texture_idx] panics when out of range.
        if (mesh_tex[m] < 0 || (uint64_t)mesh_tex[m] >= nmat) return -OR_E_INVALID;
        mesh.tris.assign(tris + 9 * off, tris + 9 * (off + mesh_ntri[m]));
        for (uint64_t t = 0; t < mesh_ntri[m]; t++) {
            const uint32_t* q = tris + 9 * (off + t);
            // mesh.rs:46-48 asserts every gathered index is in range.
            for (int k = 0; k < 3; k++)
                if (q[k] >= nv || q[3 + k] >= nuv || q[6 + k] >= nn) return -OR_E_INDEX;
        }
        off += mesh_ntri[m];
        if (o->textures[mesh.texture_idx].alpha < 1.0f)
            o->transparent.push_back(mesh);
        else
            o->opaque.push_back(mesh);
    }
    c->objects.push_back(o);
    return (int32_t)c->objects.size() - 1;
}

int32_t or_scene_new(or_ctx* c, uint64_t width, uint64_t height) {  // scene/mod.rs:760-786
    Scene s;
    s.width = width;
    s.height = height;
    Vec3 pos = V3(0.0f, 0.0f, 150.0f);
    Vec3 dir = pos * -1.0f;
    s.lights.push_back(V3(0.0f, 300.0f, 300.0f));
    float ratio = (float)width / (float)height;
    int e = camera_new(s.camera, pos, dir, ratio, -10.0f, -10.0f - 500.0f, 135.0f);
    if (e) return -e;
    c->scenes.push_back(s);
    return (int32_t)c->scenes.size() - 1;
}

int32_t or_scene_add_obj(or_ctx* c, int32_t scene, int32_t object) {
    if (scene < 0 || (size_t)scene >= c->scenes.size() || object < 0 || (size_t)object >= c->objects.size())
        return -OR_E_INVALID;
    c->scenes[scene].objects.push_back(object);
    return (int32_t)c->scenes[scene].objects.size() - 1;
}

int32_t or_scene_set_camera(or_ctx* c, int32_t scene, const float pos[3], const float dir[3], float ratio,
                            float near_, float far_, float fov_x_deg) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    return -camera_new(c->scenes[scene].camera, V3(pos[0], pos[1], pos[2]), V3(dir[0], dir[1], dir[2]), ratio, near_,
                       far_, fov_x_deg);
}

int32_t or_scene_set_lights(or_ctx* c, int32_t scene, const float* pos, uint32_t n) {
    if (scene < 0 || (size_t)scene >= c->scenes.size() || n == 0 || n > OR_MAX_LIGHTS) return -OR_E_INVALID;
    auto& s = c->scenes[scene];
    s.lights.clear();
    for (uint32_t i = 0; i < n; i++) s.lights.push_back(V3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    return OR_OK;
}

int32_t or_scene_set_interpolation(or_ctx* c, int32_t scene, int32_t mode) {
    if (scene < 0 || (size_t)scene >= c->scenes.size() || mode < 0 || mode > 1) return -OR_E_INVALID;
    c->scenes[scene].interpolation = mode;
    return OR_OK;
}

int32_t or_texmap_set_filter(or_ctx* c, int32_t texmap, int32_t filter) {
    if (texmap < 0 || (size_t)texmap >= c->texmaps.size() || filter < 0 || filter > 1) return -OR_E_INVALID;
    c->texmaps[texmap]->filter = filter;
    return OR_OK;
}

int32_t or_scene_set_exponent(or_ctx* c, int32_t scene, int32_t exponent) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    c->scenes[scene].exponent = exponent;
    return OR_OK;
}

int32_t or_scene_camera_op(or_ctx* c, int32_t scene, int32_t op, const float* v) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    Scene& s = c->scenes[scene];
    Camera& cam = s.camera;
    switch (op) {
        case 0: cam.position = cam.position + cam.up * v[0]; break;            // move_up :381-383
        case 1: cam.position = cam.position + cam.up * (-v[0]); break;         // move_down :385-387
        case 2: cam.position = cam.position + cam.u * (-v[0]); break;          // move_left :389-391
        case 3: cam.position = cam.position + cam.u * v[0]; break;             // move_right :393-395
        case 4: cam.position = cam.position + cam.up.cross(cam.u).normalized() * v[0]; break;  // :397-400
        case 5: cam.position = cam.position + cam.u.cross(cam.up).normalized() * v[0]; break;  // :402-405
        case 6: {                                                                // rotate_origin :407-413
            const float RADS_PER_DEG = 3.14159265358979323846f / 180.0f;
            Matrix4 r = Matrix4::rotate_y(v[0] * RADS_PER_DEG);
            Vec4 np = r * as_vec4(cam.position);
            Matrix4 r2 = Matrix4::rotate_y(v[0] * RADS_PER_DEG);
            Vec4 nd = r2 * as_vec4(cam.direction);
            cam.position = V3(np.a[0], np.a[1], np.a[2]);
            cam.direction = V3(nd.a[0], nd.a[1], nd.a[2]);
            break;
        }
        case 7: cam.position = V3(v[0], v[1], v[2]); break;                     // set_pos :377-379
        case 8: {                                                                // move_camera_direction :803-813
            int32_t dx = (int32_t)v[0], dy = (int32_t)v[1];
            if (!((int64_t)dx < (int64_t)s.width) || !((int64_t)dy < (int64_t)s.height)) return -OR_E_INVALID;
            float fx = (float)dx / (float)s.width, fy = (float)dy / (float)s.height;
            cam.direction = (cam.direction + cam.u * fx + cam.v * fy).normalized();  // :430-432
            update_basis(cam);
            break;
        }
        default: return -OR_E_INVALID;
    }
    return OR_OK;
}

int32_t or_scene_get_camera(or_ctx* c, int32_t scene, float pos[3], float dir[3]) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    const Camera& cam = c->scenes[scene].camera;
    for (int i = 0; i < 3; i++) {
        pos[i] = cam.position.a[i];
        dir[i] = cam.direction.a[i];
    }
    return OR_OK;
}

static int gen_transformation_matrix(Scene& s, Matrix4& M) {  // scene/mod.rs:817-899
    float n_x = (float)s.width, n_y = (float)s.height;
    Camera& cam = s.camera;
    float n = cam.min_view_dist, f = cam.max_view_dist;
    float r = cam.right, l = cam.left, t = cam.top, b = cam.bottom;
    Matrix4 mc;
    int e = gen_matrix(cam, mc);
    if (e) return e;
    Matrix4 persp = Matrix4::zeros();
    persp.a[0][0] = n;
    persp.a[1][1] = n;
    persp.a[2][2] = (n + f);
    persp.a[2][3] = -(n * f);
    persp.a[3][2] = 1.0f;
    Matrix4 orth = Matrix4::zeros();
    orth.a[0][0] = 2.0f / (r - l);
    orth.a[0][3] = -(r + l) / (r - l);
    orth.a[1][1] = 2.0f / (t - b);
    orth.a[1][3] = -(t + b) / (t - b);
    orth.a[2][2] = 2.0f / (n - f);
    orth.a[2][3] = -(n + f) / (n - f);
    orth.a[3][3] = 1.0f;
    Matrix4 vp = Matrix4::zeros();
    vp.a[0][0] = n_x / 2.0f;
    vp.a[0][3] = (n_x - 1.0f) / 2.0f;
    vp.a[1][1] = n_y / 2.0f;
    vp.a[1][3] = (n_y - 1.0f) / 2.0f;
    vp.a[2][2] = 1.0f;
    vp.a[3][3] = 1.0f;
    M = ((vp * orth) * persp) * mc;
    return OR_OK;
}

int32_t or_scene_frame_setup(or_ctx* c, int32_t scene, float Mout[16], float planes_out[24]) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    Scene& s = c->scenes[scene];
    Matrix4 M;
    int e = gen_transformation_matrix(s, M);
    if (e) return -e;
    ViewPlane pl[6];
    e = gen_view_planes(s.camera, pl);
    if (e) return -e;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) Mout[4 * i + j] = M.a[i][j];
    for (int p = 0; p < 6; p++) {
        for (int k = 0; k < 3; k++) planes_out[4 * p + k] = pl[p].normal.a[k];
        planes_out[4 * p + 3] = pl[p].k;
    }
    return OR_OK;
}

int32_t or_canvas_new(or_ctx* c, uint64_t width, uint64_t height) {  // canvas.rs:366-380
    if (width == 0 || height == 0) return -OR_E_INVALID;
    Canvas cv;
    cv.width = width;
    cv.height = height;
    cv.frame.assign(width * height, pixel_new(0, 0, 0));
    c->canvases.push_back(cv);
    return (int32_t)c->canvases.size() - 1;
}

static Canvas* get_canvas(or_ctx* c, int32_t i) {
    if (i < 0 || (size_t)i >= c->canvases.size()) return nullptr;
    return &c->canvases[i];
}

int32_t or_canvas_init_depth(or_ctx* c, int32_t canvas, float depth) {
    Canvas* cv = get_canvas(c, canvas);
    if (!cv) return -OR_E_INVALID;
    cv->init_depth(depth);
    return OR_OK;
}

int32_t or_canvas_apply_offset(or_ctx* c, int32_t canvas, int32_t x, int32_t y) {  // canvas.rs:382-385
    Canvas* cv = get_canvas(c, canvas);
    if (!cv) return -OR_E_INVALID;
    cv->offset.x = (float)x;
    cv->offset.y = (float)y;
    return OR_OK;
}

int32_t or_canvas_resize(or_ctx* c, int32_t canvas, uint64_t width, uint64_t height) {  // canvas.rs:387-393
    Canvas* cv = get_canvas(c, canvas);
    if (!cv || width == 0 || height == 0) return -OR_E_INVALID;
    cv->width = width;
    cv->height = height;
    cv->frame.resize(width * height, pixel_new(0, 0, 0));
    cv->init_depth(cv->depth_max);
    return OR_OK;
}

int32_t or_canvas_clear(or_ctx* c, int32_t canvas) {
    Canvas* cv = get_canvas(c, canvas);
    if (!cv) return -OR_E_INVALID;
    cv->clear();
    return OR_OK;
}

int32_t or_canvas_read(or_ctx* c, int32_t canvas, uint8_t* bgra, float* depth) {
    Canvas* cv = get_canvas(c, canvas);
    if (!cv) return -OR_E_INVALID;
    if (bgra) std::memcpy(bgra, cv->frame.data(), cv->frame.size() * 4);
    if (depth) {
        if (cv->depth_frame.size() != cv->frame.size()) return -OR_E_DEPTH_UNINIT;
        std::memcpy(depth, cv->depth_frame.data(), cv->depth_frame.size() * 4);
    }
    return OR_OK;
}

int32_t or_canvas_write(or_ctx* c, int32_t canvas, const uint8_t* bgra, const float* depth) {
    Canvas* cv = get_canvas(c, canvas);
    if (!cv) return -OR_E_INVALID;
    if (bgra) std::memcpy(cv->frame.data(), bgra, cv->frame.size() * 4);
    if (depth) {
        if (cv->depth_frame.size() != cv->frame.size()) return -OR_E_DEPTH_UNINIT;
        std::memcpy(cv->depth_frame.data(), depth, cv->depth_frame.size() * 4);
    }
    return OR_OK;
}

// Builds the VertexAttributes triple of scene/mod.rs:933-1014 for one indexed triangle.
static void assemble(const Object& o, const uint32_t* q, const std::vector<Attr>& vis, Triangle& t, int nl) {
    for (int k = 0; k < 3; k++) {
        uint32_t vi = q[k], ti = q[3 + k], ni = q[6 + k];
        t.v[k] = o.vertices[vi];
        Attr& a = t.at[k];
        a = vis[vi];
        a.screen_coord = Vec2{0.0f, 0.0f};
        a.normal = o.normals[ni];
        a.texture_coord = o.uvs[ti];
        (void)nl;
    }
}

// Projection of one clipped triangle and its draw call, scene/mod.rs:1047-1083.
static void project_and_draw(Canvas& cv, const Matrix4& M, Triangle& ct, const Texture& tex, int nl, int exponent,
                             int interp) {
    float ws[3];
    for (int k = 0; k < 3; k++) {
        Vec4 p = M * as_vec4(ct.v[k]);
        float w = p.a[3];
        ws[k] = w;
        ct.at[k].screen_coord = Vec2{p.a[0], p.a[1]} / w;
    }
    draw_triangle_with_attributes(cv, ct.at[0], ct.at[1], ct.at[2], tex, nl, exponent, ws, interp);
}

// Scene::render, scene/mod.rs:901-1249.
int32_t or_scene_render(or_ctx* c, int32_t scene, int32_t canvas) {
    if (scene < 0 || (size_t)scene >= c->scenes.size()) return -OR_E_INVALID;
    Canvas* cvp = get_canvas(c, canvas);
    if (!cvp) return -OR_E_INVALID;
    Canvas& cv = *cvp;
    if (cv.depth_frame.size() != cv.frame.size()) return -OR_E_DEPTH_UNINIT;
    Scene& s = c->scenes[scene];
    int nl = (int)s.lights.size();
    cv.err = OR_OK;
    cv.clear();
    Matrix4 M;
    int e = gen_transformation_matrix(s, M);
    if (e) return -e;
    Vec3 cam = s.camera.position;
    ViewPlane planes[6];
    e = gen_view_planes(s.camera, planes);
    if (e) return -e;
    Triangle clipped[12];
    Texture deflt = texture_default();
    for (int32_t oid : s.objects) {
        Object& o = *c->objects[oid];
        // per-vertex visual info, scene/mod.rs:917-926
        std::vector<Attr> vis(o.vertices.size());
        for (size_t i = 0; i < o.vertices.size(); i++) {
            Vec3 v = o.vertices[i];
            Vec3 eye_dir = v - cam;
            Vec3 eye = eye_dir.normalized();
            vis[i].depth = eye_dir.norm();
            for (int l = 0; l < nl; l++) {
                vis[i].light[l] = (v - s.lights[l]).normalized();
                vis[i].halfway[l] = (vis[i].light[l] + eye).normalized();
            }
        }
        cv.depth_update_enabled = true;
        for (const Mesh& m : o.opaque) {
            const Texture& tex = (size_t)m.texture_idx < o.textures.size() ? o.textures[m.texture_idx] : deflt;
            size_t nt = m.tris.size() / 9;
            for (size_t ti = 0; ti < nt; ti++) {
                Triangle t;
                assemble(o, &m.tris[9 * ti], vis, t, nl);
                Vec3 n = calc_normal(t);
                Vec3 tri_eye = cam - get_center(t);
                if (tri_eye.dot(n) <= 0.0f) continue;  // back-face culling, :1016-1027
                int cnt = clip_against_planes(t, planes, clipped, nl);
                for (int k = 0; k < cnt; k++) {
                    project_and_draw(cv, M, clipped[k], tex, nl, s.exponent, s.interpolation);
                    if (cv.err) return -cv.err;
                }
            }
        }
        cv.depth_update_enabled = false;
        for (Mesh& m : o.transparent) {
            const Texture& tex = (size_t)m.texture_idx < o.textures.size() ? o.textures[m.texture_idx] : deflt;
            size_t nt = m.tris.size() / 9;
            // painter's sort, scene/mod.rs:1100-1115: stable, descending total order of the distance
            std::vector<std::pair<uint32_t, size_t>> key(nt);
            for (size_t ti = 0; ti < nt; ti++) {
                const uint32_t* q = &m.tris[9 * ti];
                Vec3 ctr = (o.vertices[q[0]] + o.vertices[q[1]] + o.vertices[q[2]]) / 3.0f;
                float d = (ctr - cam).norm();
                uint32_t bits;
                std::memcpy(&bits, &d, 4);
                bits = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);  // total_cmp order
                key[ti] = {bits, ti};
            }
            std::stable_sort(key.begin(), key.end(),
                             [](const std::pair<uint32_t, size_t>& a, const std::pair<uint32_t, size_t>& b) {
                                 return a.first > b.first;
                             });
            std::vector<uint32_t> sorted(m.tris.size());
            for (size_t ti = 0; ti < nt; ti++)
                std::memcpy(&sorted[9 * ti], &m.tris[9 * key[ti].second], 9 * sizeof(uint32_t));
            m.tris.swap(sorted);
            for (size_t ti = 0; ti < nt; ti++) {
                Triangle t;
                assemble(o, &m.tris[9 * ti], vis, t, nl);
                int cnt = clip_against_planes(t, planes, clipped, nl);
                for (int k = 0; k < cnt; k++) {
                    project_and_draw(cv, M, clipped[k], tex, nl, s.exponent, s.interpolation);
                    if (cv.err) return -cv.err;
                }
            }
        }
    }
    return OR_OK;
}

int32_t or_object_transparent_tris(or_ctx* c, int32_t object, uint32_t mesh, uint32_t* out, uint64_t cap) {
    if (object < 0 || (size_t)object >= c->objects.size()) return -OR_E_INVALID;
    Object& o = *c->objects[object];
    if (mesh >= o.transparent.size()) return -OR_E_INVALID;
    const auto& t = o.transparent[mesh].tris;
    if (cap < t.size()) return -OR_E_INVALID;
    std::memcpy(out, t.data(), t.size() * 4);
    return (int32_t)(t.size() / 9);
}

// Canvas::draw_triangle, canvas.rs:435-575 (the GUI's 2D textured, alpha-blended triangle).
int32_t or_canvas_draw_triangle_2d(or_ctx* c, int32_t canvas, const float vv[24], int32_t texmap,
                                   const uint64_t* clip) {
    Canvas* cvp = get_canvas(c, canvas);
    if (!cvp) return -OR_E_INVALID;
    Canvas& cv = *cvp;
    if (cv.depth_frame.size() != cv.frame.size()) return -OR_E_DEPTH_UNINIT;
    if (texmap < 0 || (size_t)texmap >= c->texmaps.size()) return -OR_E_INVALID;  // :444-447 assert
    const TextureMap& dm = *c->texmaps[texmap];
    Vec2 ctr[3], uv[3];
    Pixel col[3];
    float al[3];
    for (int k = 0; k < 3; k++) {
        const float* p = vv + 8 * k;
        ctr[k] = cv.pos_map_center(Vec2{p[0], p[1]});
        uv[k] = Vec2{p[2], p[3]};
        col[k] = pixel_new((uint8_t)p[4], (uint8_t)p[5], (uint8_t)p[6]);
        al[k] = p[7];
    }
    Vec2 a = ctr[0], b = ctr[1], cc = ctr[2];
    uint64_t x_min = as_usize(min3(a.x, b.x, cc.x));
    uint64_t y_min = as_usize(min3(a.y, b.y, cc.y));
    uint64_t x_max = as_usize(max3(a.x, b.x, cc.x));
    uint64_t y_max = as_usize(max3(a.y, b.y, cc.y));
    Rect drawable = Rect::from_coords(x_min, y_min, x_max, y_max);
    Rect screen = Rect::from_coords(0, 0, cv.width - 1, cv.height - 1);
    drawable = Rect::clip(drawable, screen);
    Rect cr = clip ? Rect::from_coords(clip[0], clip[1], clip[2], clip[3]) : screen;
    Rect valid = Rect::clip(cr, drawable);
    x_min = valid.x_min();
    y_min = valid.y_min();
    x_max = valid.x_max();
    y_max = valid.y_max();
    float f_alpha = edge(b, cc, a.x, a.y);
    float f_beta = edge(cc, a, b.x, b.y);
    float f_gama = edge(a, b, cc.x, cc.y);
    float f_alpha_out = edge(b, cc, -1.0f, -1.0f);
    float f_beta_out = edge(cc, a, -1.0f, -1.0f);
    float f_gama_out = edge(a, b, -1.0f, -1.0f);
    for (uint64_t y = y_min; y <= y_max; y++) {
        float yf = (float)y;
        for (uint64_t x = x_min; x <= x_max; x++) {
            float xf = (float)x;
            float alpha = edge(b, cc, xf, yf) / f_alpha;
            float beta = edge(cc, a, xf, yf) / f_beta;
            float gama = edge(a, b, xf, yf) / f_gama;
            if (!(alpha >= 0.0f && beta >= 0.0f && gama >= 0.0f)) continue;
            if (!((alpha > 0.0f || f_alpha * f_alpha_out > 0.0f) && (beta > 0.0f || f_beta * f_beta_out > 0.0f) &&
                  (gama > 0.0f || f_gama * f_gama_out > 0.0f)))
                continue;
            Pixel cp = pixel_add(pixel_add(pixel_mul(col[0], alpha), pixel_mul(col[1], beta)), pixel_mul(col[2], gama));
            float calpha = (alpha * al[0]) + (beta * al[1]) + (gama * al[2]);
            Vec2 cuv = (uv[0] * alpha) + (uv[1] * beta) + (uv[2] * gama);
            uint8_t rgba[4];
            if (!get_rgba_slice(dm, cuv.x, cuv.y, rgba)) return -OR_E_TEXTURE_RANGE;
            float talpha = (float)rgba[3] / 255.0f;
            Pixel ct = pixel_new(rgba[0], rgba[1], rgba[2]);
            cp = pixel_add(pixel_mul(cp, talpha), pixel_mul(ct, 1.0f - talpha));
            float fa = calpha * talpha;
            cv.draw_pixel_coord_with_depth(x, y, cp, fa, 0.0f);
        }
    }
    return OR_OK;
}

}  // extern "C"
