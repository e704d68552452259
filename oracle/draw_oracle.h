/*
 * draw_oracle.h -- CPU restatement of the draw renderer's hot path (TEST INFRASTRUCTURE).
 *
 * This is the parity oracle. It is not part of the product: only tests/, the
 * smoke check in __graft_entry__.py and the CPU-baseline leg of bench.py load it,
 * and only as the checker or as the timed CPU baseline.
 *
 * It restates, expression for expression and in the same evaluation order, the
 * reference renderer written in Rust (mororo18/draw):
 *   src/renderer/linalg.rs           Vec2/Vec3/Vec4/Matrix4
 *   src/renderer/canvas.rs           Canvas, Pixel, VertexAttributes, Rectangle,
 *                                    draw_triangle_with_attributes, draw_triangle
 *   src/renderer/scene/mod.rs        Camera, ViewPlane, Triangle clipping,
 *                                    TextureMap, Texture, Scene::render
 *   src/renderer/scene/mesh.rs       IndexedMesh gathers
 *   src/renderer/scene/object.rs     Object::new (opaque / transparent split)
 *
 * Parity status: UNPINNED by the reference itself. The reference ships no
 * tests, golden vectors or fixtures, and it cannot be compiled here (it is Rust
 * with un-vendored git dependencies and X11 linkage, and no Rust toolchain is
 * installed). The restatement is cross-checked against hand-derived
 * known-answer cases and against an independent pure-Python restatement.
 *
 * Build: g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fPIC -shared
 * (-ffp-contract=off matters on aarch64, where GCC would otherwise fuse
 * mul+add into FMA; Rust never contracts.)
 *
 * Extensions beyond the reference (all default to the reference's constants):
 * camera near/far/fov_x, N point lights (per-light terms summed in light
 * order; with one light the formula is the reference's), an integer specular
 * exponent (reference: 2), and the depth clear value.
 */
#ifndef DRAW_ORACLE_H
#define DRAW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes; same numeric values as the product's DG_* codes. */
#define OR_OK 0
#define OR_E_INVALID 1        /* bad argument (reference: assert!/unwrap panic) */
#define OR_E_INDEX 2          /* mesh index out of range (mesh.rs:46-48 assert) */
#define OR_E_TEXTURE_RANGE 3  /* texel offset outside the image (slice index panic) */
#define OR_E_CAMERA 4         /* camera / view-plane assertion (scene/mod.rs:327-331, 420, 624) */
#define OR_E_DEPTH_UNINIT 5   /* render before init_depth (canvas.rs:914 debug_assert) */

#define OR_MAX_LIGHTS 8

/* Material: the reference's `Texture` (scene/mod.rs:206-216). map_* = texture
 * map handle, or -1 for the 1x1 white default (scene/mod.rs:128-135). */
typedef struct {
    float ka[3];
    float kd[3];
    float ks[3];
    float alpha;
    int32_t map_ka;
    int32_t map_kd;
} or_material;

typedef struct or_ctx or_ctx;

or_ctx* or_ctx_new(void);
void or_ctx_free(or_ctx* c);

/* TextureMap::new(img, width, height, components), scene/mod.rs:113-126. Returns handle >= 0 or -code. */
int32_t or_texmap_new(or_ctx* c, const uint8_t* img, uint64_t len, uint64_t w, uint64_t h, uint64_t comps);

/* Object::new, object.rs:34-71. vertices/normals/uvs are Vec3 lists (3 floats each).
 * tris: 9 indices per triangle in the reference's tuple order
 * (position[3], texture[3], normal[3]), meshes concatenated; mesh_ntri[i] triangles
 * for mesh i, whose texture (material) index is mesh_tex[i]. Returns handle or -code. */
int32_t or_object_new(or_ctx* c, const float* vertices, uint64_t nv, const float* normals, uint64_t nn,
                      const float* uvs, uint64_t nuv, const uint32_t* tris, const uint64_t* mesh_ntri,
                      const int32_t* mesh_tex, uint64_t nmesh, const or_material* mats, uint64_t nmat);

/* Scene::new(width, height), scene/mod.rs:760-786. Returns handle or -code. */
int32_t or_scene_new(or_ctx* c, uint64_t width, uint64_t height);
int32_t or_scene_add_obj(or_ctx* c, int32_t scene, int32_t object);
/* Camera::new(pos, dir, ratio) with the projection constants made explicit
 * (reference: near=-10, far=near-500, fov_x=135, scene/mod.rs:308-310). */
int32_t or_scene_set_camera(or_ctx* c, int32_t scene, const float pos[3], const float dir[3], float ratio,
                            float near_, float far_, float fov_x_deg);
int32_t or_scene_set_lights(or_ctx* c, int32_t scene, const float* pos, uint32_t n);
int32_t or_scene_set_exponent(or_ctx* c, int32_t scene, int32_t exponent);
/* Extensions without a counterpart in the reference (defaults = the reference):
 * interpolation of the shading attributes (OR_INTERP_AFFINE: the reference's
 * screen-space barycentrics; OR_INTERP_PERSPECTIVE: weighted by 1/w, see
 * draw_triangle_with_attributes) and a texture map's filter (OR_FILTER_NEAREST:
 * get_rgb_slice; OR_FILTER_BILINEAR: get_rgb_bilinear). */
#define OR_INTERP_AFFINE 0
#define OR_INTERP_PERSPECTIVE 1
#define OR_FILTER_NEAREST 0
#define OR_FILTER_BILINEAR 1
int32_t or_scene_set_interpolation(or_ctx* c, int32_t scene, int32_t mode);
int32_t or_texmap_set_filter(or_ctx* c, int32_t texmap, int32_t filter);
/* Camera movement, scene/mod.rs:377-413, 430-432, 803-813. op: 0 up,1 down,2 left,3 right,4 foward,5 backward,
 * 6 rotate_origin(deg), 7 set_pos(v3), 8 move_camera_direction(dx,dy as ints in v[0],v[1]). */
int32_t or_scene_camera_op(or_ctx* c, int32_t scene, int32_t op, const float* v);
int32_t or_scene_get_camera(or_ctx* c, int32_t scene, float pos[3], float dir[3]);

/* Per-frame host setup (scene/mod.rs:817-899, 481-593): the transformation
 * matrix (row-major 16 floats) and the 6 planes (near, far, right, left, top,
 * bottom; 4 floats each: normal xyz, k). Mutates the camera basis like render. */
int32_t or_scene_frame_setup(or_ctx* c, int32_t scene, float M[16], float planes[24]);

/* Canvas (canvas.rs:353-433). */
int32_t or_canvas_new(or_ctx* c, uint64_t width, uint64_t height);
int32_t or_canvas_init_depth(or_ctx* c, int32_t canvas, float depth);
int32_t or_canvas_apply_offset(or_ctx* c, int32_t canvas, int32_t x, int32_t y);
int32_t or_canvas_resize(or_ctx* c, int32_t canvas, uint64_t width, uint64_t height);
int32_t or_canvas_clear(or_ctx* c, int32_t canvas);
/* Copies out the BGRA frame (as_bytes_slice, canvas.rs:974-978) and the depth buffer. */
int32_t or_canvas_read(or_ctx* c, int32_t canvas, uint8_t* bgra, float* depth);
int32_t or_canvas_write(or_ctx* c, int32_t canvas, const uint8_t* bgra, const float* depth);

/* Scene::render(&mut canvas), scene/mod.rs:901-1249. */
int32_t or_scene_render(or_ctx* c, int32_t scene, int32_t canvas);

/* Reads back the (possibly re-sorted, scene/mod.rs:1100-1115) triangle order of a
 * transparent mesh: 9 indices per triangle. */
int32_t or_object_transparent_tris(or_ctx* c, int32_t object, uint32_t mesh, uint32_t* out, uint64_t cap);

/* The 2D overlay triangle (Canvas::draw_triangle, canvas.rs:435-575) used by the GUI.
 * v: 3 vertices x (screen x, screen y, u, v, r, g, b, alpha) ; clip: x0,y0,x1,y1 or NULL. */
int32_t or_canvas_draw_triangle_2d(or_ctx* c, int32_t canvas, const float v[24], int32_t texmap,
                                   const uint64_t* clip);

#ifdef __cplusplus
}
#endif
#endif
