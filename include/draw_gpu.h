/*
 * draw_gpu.h -- C ABI of the GB300 (sm_103a) rasterizer that replaces the CPU
 * draw call of the reference renderer (mororo18/draw, Rust).
 *
 * The reference's boundary is `Scene::render(&mut self, canvas: &mut Canvas)`
 * (src/renderer/scene/mod.rs:901) with its supporting object model. Each entry
 * point below names the reference item it replaces. All functions return a
 * dg_status (0 = DG_OK) and never abort; conditions on which the reference
 * panics (assert!, unwrap, slice index) come back as error codes.
 *
 * Threading: one dg_ctx may be used by one host thread at a time
 * (thread-compatible, like the reference's &mut Scene / &mut Canvas).
 * Resources (texture maps, objects, scenes, canvases) are int32 ids owned by
 * their context. Device work is enqueued on the context's CUDA stream; calls
 * that hand data back to the host synchronize that stream.
 *
 * Colour buffers keep the reference's memory layout: BGRA bytes (Pixel,
 * canvas.rs:51-59), row 0 = top of the screen (canvas.rs:941-942). Depth is
 * f32 indexed y*W+x with y = 0 at the bottom (canvas.rs:413-423).
 */
#ifndef DRAW_GPU_H
#define DRAW_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t dg_status;
#define DG_OK 0
#define DG_E_INVALID 1        /* bad argument; the reference panics (assert!/unwrap) */
#define DG_E_INDEX 2          /* mesh index out of range (scene/mesh.rs:46-48 assert) */
#define DG_E_TEXTURE_RANGE 3  /* texel offset outside the image (scene/mod.rs:151,167 slice index) */
#define DG_E_CAMERA 4         /* camera / view-plane assertion (scene/mod.rs:327-331, 420, 624) */
#define DG_E_DEPTH_UNINIT 5   /* render before init_depth (canvas.rs:914 debug_assert) */
#define DG_E_CUDA 6           /* CUDA runtime error */
#define DG_E_OOM 7            /* device memory exhausted or over budget */
#define DG_E_LIMIT 8          /* size beyond a documented limit */
#define DG_E_TIMEOUT 9        /* a bounded wait gave up */
#define DG_E_CANCELLED 10     /* a render-server request cancelled before it was admitted */

#define DG_MAX_LIGHTS 8

/* Extensions without a counterpart in the reference (the defaults are the
 * reference's behaviour): how a scene interpolates its shading attributes and
 * how a texture map is sampled. */
#define DG_INTERP_AFFINE 0       /* screen-space barycentrics (canvas.rs:682-722) */
#define DG_INTERP_PERSPECTIVE 1  /* perspective-correct: weighted by 1/w */
#define DG_FILTER_NEAREST 0      /* nearest texel (scene/mod.rs:154-168) */
#define DG_FILTER_BILINEAR 1     /* bilinear blend of four texels */

typedef struct dg_ctx dg_ctx;

/* Material: the reference's `Texture` (scene/mod.rs:206-216). map_ka/map_kd are
 * texture-map ids from dg_texmap_create, or -1 for the 1x1 white default map
 * (TextureMap::default, scene/mod.rs:128-135). */
typedef struct {
    float ka[3];
    float kd[3];
    float ks[3];
    float alpha;
    int32_t map_ka;
    int32_t map_kd;
} dg_material;

/* One IndexedMesh (scene/mesh.rs:30-35): ntri triangles of 9 indices each in the
 * reference's tuple order (position[3], texture[3], normal[3]; object.rs:431-434),
 * drawn with material texture_idx of its object. */
typedef struct {
    const uint32_t* tris;
    uint64_t ntri;
    int32_t texture_idx;
} dg_mesh_desc;

/* ------------------------------------------------------------------ context */
/* device >= 0: a CUDA device. device == -1: a host-only context in which scenes,
 * cameras and dg_scene_frame_setup work and every device call returns DG_E_CUDA. */
dg_status dg_ctx_create(int32_t device, dg_ctx** out);
dg_status dg_ctx_destroy(dg_ctx* ctx);
const char* dg_status_string(dg_status s);
/* Waits for the context stream and returns (and clears) any error the kernels raised. */
dg_status dg_ctx_synchronize(dg_ctx* ctx);
/* Replaces the context's stream (cudaStream_t passed as void*; NULL = own stream). */
dg_status dg_ctx_set_stream(dg_ctx* ctx, void* stream);
void* dg_ctx_stream(dg_ctx* ctx);
/* Per-kernel CUDA-event timing of the last render (ms), up to 5 values: "vertex", "cull",
 * "setup_raster", "queue_raster", "resolve". Enabled with dg_ctx_set_timing(ctx, 1); the
 * events between kernels also stop their launch overlap, so frames are slower meanwhile. */
dg_status dg_ctx_set_timing(dg_ctx* ctx, int32_t enable);
dg_status dg_ctx_kernel_times(dg_ctx* ctx, float* ms, int32_t n);
/* Kernel timeline of the render jobs since the last call, in builds made with
 * DRAW_TIMELINE (draw_gb300/_build.py build(timeline=True)); other builds
 * return DG_E_INVALID. out[4k .. 4k+3] for kernel k in the order of
 * dg_ctx_kernel_times: the global timer (ns) when its first block started, when
 * its first and its last block passed the wait for the previous kernel, and
 * when its last block finished; 0 where nothing was recorded (a kernel that did
 * not run; a resolve pass whose tiles were all cleared before the wait).
 * Synchronizes the context's stream and clears the record. */
dg_status dg_timeline_read(dg_ctx* ctx, uint64_t* out, int32_t n);
/* Launch-shape knobs of the raster passes (chosen by dg_autotune below):
 * small_max_px: triangles whose clipped bounding box has at most this many
 * pixels are rasterized one triangle per lane, the others are cut into 32-pixel
 * units spread over all warps (0 = all cut into units, max 4096;
 * DG_SMALL_MAX_PX_AUTO, the default: per frame, 64 when the frame has at least
 * as many triangles as pixels, else 16); setup_blocks_per_sm,
 * queue_blocks_per_sm and cull_blocks_per_sm: grid sizes (caps) of those
 * passes in 256-thread blocks per SM (1..64); record_limit: 0, or at most this
 * many triangle records per render (triangles beyond it are shaded from the
 * mesh again in the resolve pass); tile_rows: height of the resolve pass's
 * 32-pixel-wide tiles (8, 16 or 32; 0, the default: per render job, the tallest
 * whose tiles fill 4 resolve blocks per SM, else 8); item_units: 32-pixel units per work item
 * of the queue pass (1..256). Results do not depend on them. */
#define DG_SMALL_MAX_PX_AUTO 0xFFFFFFFFu
typedef struct {
    uint32_t small_max_px;
    uint32_t setup_blocks_per_sm;
    uint32_t queue_blocks_per_sm;
    uint32_t cull_blocks_per_sm;
    uint32_t record_limit;
    uint32_t tile_rows;
    uint32_t item_units;
} dg_tuning;
dg_status dg_ctx_set_tuning(dg_ctx* ctx, const dg_tuning* t);
dg_status dg_ctx_get_tuning(dg_ctx* ctx, dg_tuning* t);

/* Counters of the last render (up to 14): [0] vertices, [1] input triangles, [2] triangles
 * queued for the load-balanced raster pass, [3] their 32-pixel work units, [4] covered
 * pixels (written by resolve), [5] triangles rasterized in place because the queue, the
 * small-triangle list or the triangle records were full, [6] host-to-device bytes of the
 * job descriptor, [7] kernels launched, [8] triangles that passed the cull pass,
 * [9] triangles (clip outputs counted one by one) that asked for a triangle record, [10] light/halfway rows handed out to clip vertices,
 * [11] triangles on the small-triangle list, [12] the resolve tile height the job used,
 * [13] the small-triangle threshold of its first frame. Synchronizes. */
dg_status dg_ctx_last_stats(dg_ctx* ctx, uint64_t* out, int32_t n);

/* Self-check of the division the raster pass uses for the barycentrics of a
 * covered pixel: a / b computed from the reciprocal RN(1/b) by two residual
 * corrections (Markstein's method) must equal IEEE a / b bit for bit. Checks
 * `samples` seeded pairs (a, b) and (-a, b) of one family on the device:
 * mode 0 every integer pair 0 <= a <= b <= 4096, mode 1 integers b <= 2^24 and
 * a <= b, mode 2 integer-valued b < 2^101 and a < 4b, mode 3 a < 2^61 and
 * b < 2^100 with random mantissas. Writes the mismatch count and, when there is
 * one, the first mismatching pair seen. Synchronizes. */
dg_status dg_check_division(dg_ctx* ctx, int32_t mode, uint64_t samples, uint64_t seed, uint64_t* mismatches,
                            float* first_a, float* first_b);

/* -------------------------------------------------------------- texture map */
/* TextureMap::new(img, width, height, components), scene/mod.rs:113-126. */
dg_status dg_texmap_create(dg_ctx* ctx, const uint8_t* img, uint64_t len, uint64_t width, uint64_t height,
                           uint64_t components, int32_t* out_id);
/* Extension, no counterpart in the reference (TextureMap::get_rgb_slice,
 * scene/mod.rs:154-168, samples the nearest texel): DG_FILTER_BILINEAR blends
 * four texels. x = u*(W-1), y = v*(H-1); the base texel (floor x, floor y) has
 * the nearest texel's offset; the others are the next column (the same one at
 * the last column) and the next row up (the same one at the top row). With
 * c = byte/255, ax = x - floor x, ay = y - floor y, per channel:
 * t0 = c00*(1-ax) + c01*ax, t1 = c10*(1-ax) + c11*ax, c = t0*(1-ay) + t1*ay.
 * An offset past the image is DG_E_TEXTURE_RANGE. Default DG_FILTER_NEAREST. */
dg_status dg_texmap_set_filter(dg_ctx* ctx, int32_t texmap, int32_t filter);

/* ------------------------------------------------------------------- object */
/* Object::new(name, vertices, normals, texture_vertices, meshes, textures),
 * object.rs:34-71. vertices/normals/uvs are Vec3 lists (3 floats each; the
 * reference stores UVs as Vec3 with z = 0, object.rs:151-155). Meshes whose
 * material alpha < 1 form the transparent pass (object.rs:45-53). Indices are
 * validated here (the reference asserts them during render). */
dg_status dg_object_create(dg_ctx* ctx, const float* vertices, uint64_t nv, const float* normals, uint64_t nn,
                           const float* uvs, uint64_t nuv, const dg_mesh_desc* meshes, uint64_t nmesh,
                           const dg_material* materials, uint64_t nmat, int32_t* out_id);
dg_status dg_object_destroy(dg_ctx* ctx, int32_t object);

/* ---------------------------------------------------------- OBJ/MTL loader
 * Object::load_from_file (object.rs:106-454) as a parser whose result the
 * caller turns into an object with dg_texmap_create and dg_object_create (the
 * reference decodes texture images with stb_image; this library leaves image
 * decoding to the caller and returns the map paths). The parser follows the
 * reference's use of the OBJ data: quads split as (a, b, c), (c, d, a); faces
 * of more than 4 vertices DG_E_LIMIT (the reference's todo!); normals
 * normalized; positions scaled so the largest |v| is 100; materials
 * [Texture::default(), MTL materials in library order]; one mesh per non-empty
 * group; dummy texture coordinates and generated smooth normals for groups
 * whose faces lack them. DG_E_INVALID where the reference panics (unopenable
 * file, missing Ka/Kd/Ks, a face of fewer than 3 vertices, no positions). */
typedef struct dg_obj dg_obj;
dg_status dg_obj_parse(const char* path, dg_obj** out);
/* [0] positions, [1] normals, [2] texture coordinates, [3] meshes, [4] materials, [5] triangles. */
dg_status dg_obj_counts(const dg_obj* h, uint64_t* out, int32_t n);
/* Vec3 lists (3 floats each; texture coordinates as (u, v, 0)); any pointer may be NULL. */
dg_status dg_obj_arrays(const dg_obj* h, float* vertices, float* normals, float* uvs);
/* Mesh `mesh`: its triangles (9 indices each, as dg_mesh_desc), material index and group name. */
dg_status dg_obj_mesh(const dg_obj* h, uint64_t mesh, uint32_t* tris, uint64_t cap, uint64_t* ntri,
                      int32_t* texture_idx, char* name, uint64_t name_cap);
/* Material i (0 = Texture::default()): constants (map ids set to -1), name and the map file paths
 * ("" when the material has none). */
dg_status dg_obj_material(const dg_obj* h, uint64_t i, dg_material* m, char* name, uint64_t name_cap,
                          char* map_ka, char* map_kd, uint64_t path_cap);
dg_status dg_obj_name(const dg_obj* h, char* name, uint64_t cap);
dg_status dg_obj_free(dg_obj* h);

/* -------------------------------------------------------------------- scene */
/* Scene::new(width, height), scene/mod.rs:760-786: camera at (0,0,150) looking
 * at the origin, light at (0,300,300). */
dg_status dg_scene_create(dg_ctx* ctx, uint64_t width, uint64_t height, int32_t* out_id);
/* Scene::add_obj(obj) -> ObjectInfo.id, scene/mod.rs:788-801. */
dg_status dg_scene_add_obj(dg_ctx* ctx, int32_t scene, int32_t object, uint32_t* out_obj_id);
/* Camera::new(pos, dir, ratio), scene/mod.rs:297-357, with the projection
 * constants explicit (reference: near=-10, far=-510, fov_x=135 degrees). */
dg_status dg_scene_set_camera(dg_ctx* ctx, int32_t scene, const float pos[3], const float dir[3], float ratio,
                              float near_, float far_, float fov_x_deg);
/* Camera movement: op 0 move_up, 1 move_down, 2 move_left, 3 move_right,
 * 4 move_foward, 5 move_backward (arg[0] = dist; scene/mod.rs:381-405),
 * 6 rotate_origin(arg[0] degrees; :407-413), 7 set_pos(arg[0..3]; :377-379),
 * 8 Scene::move_camera_direction(dx = arg[0], dy = arg[1]; :803-813). */
dg_status dg_scene_camera_op(dg_ctx* ctx, int32_t scene, int32_t op, const float* arg);
dg_status dg_scene_get_camera(dg_ctx* ctx, int32_t scene, float pos[3], float dir[3]);
/* Extensions (reference: one light at Scene.light_source, exponent 2 at canvas.rs:724). */
dg_status dg_scene_set_lights(dg_ctx* ctx, int32_t scene, const float* pos, uint32_t n);
dg_status dg_scene_set_exponent(dg_ctx* ctx, int32_t scene, int32_t exponent);
/* Extension, no counterpart in the reference: DG_INTERP_PERSPECTIVE interpolates
 * texture coordinates, normals and the light/halfway vectors with
 * perspective-correct weights. From the reference's screen-space barycentrics
 * alpha, beta, gama (canvas.rs:673-681) and the vertices' clip-space w (the
 * projection's divisor, scene/mod.rs:1047-1050): pa = alpha * (1/w_a),
 * pb = beta * (1/w_b), pc = gama * (1/w_c), s = (pa + pb) + pc, weights
 * pa/s, pb/s, pc/s, each attribute (a*wa + b*wb) + c*wc in f32 without
 * contraction. Coverage and depth (the interpolated eye distance) keep the
 * reference's weights, so they are identical in both modes. Default
 * DG_INTERP_AFFINE (the reference). */
dg_status dg_scene_set_interpolation(dg_ctx* ctx, int32_t scene, int32_t mode);
/* Host frame setup of Scene::render (gen_transformation_matrix, scene/mod.rs:817-899,
 * and Camera::gen_view_planes, :481-593): M row-major, planes near, far, right,
 * left, top, bottom as (normal xyz, k). Updates the camera basis like render. */
dg_status dg_scene_frame_setup(dg_ctx* ctx, int32_t scene, float M[16], float planes[24]);
/* Reads the current order of a transparent mesh's triangles (the reference
 * re-sorts them in place every frame, scene/mod.rs:1100-1115). */
dg_status dg_object_transparent_tris(dg_ctx* ctx, int32_t object, uint32_t mesh, uint32_t* out, uint64_t cap,
                                     uint64_t* out_ntri);

/* ------------------------------------------------------------------- canvas */
/* Canvas::new(width, height), canvas.rs:366-380 (frame black, depth absent). */
dg_status dg_canvas_create(dg_ctx* ctx, uint64_t width, uint64_t height, int32_t* out_id);
dg_status dg_canvas_destroy(dg_ctx* ctx, int32_t canvas);
dg_status dg_canvas_init_depth(dg_ctx* ctx, int32_t canvas, float depth);          /* canvas.rs:403-411 */
dg_status dg_canvas_apply_offset(dg_ctx* ctx, int32_t canvas, int32_t x, int32_t y); /* canvas.rs:382-385 */
dg_status dg_canvas_resize(dg_ctx* ctx, int32_t canvas, uint64_t width, uint64_t height); /* canvas.rs:387-393 */
dg_status dg_canvas_clear(dg_ctx* ctx, int32_t canvas);                            /* canvas.rs:425-433 */
/* Canvas::as_bytes_slice (canvas.rs:974-978) and the depth buffer, copied to host
 * memory (either pointer may be NULL). Synchronizes; returns kernel errors. */
dg_status dg_canvas_read(dg_ctx* ctx, int32_t canvas, uint8_t* bgra, float* depth);
/* The same copy without waiting: it starts once the work already queued on the
 * context stream has finished, and runs on a separate copy stream, so the next
 * frame (into another canvas) renders while this one is copied out. The host
 * buffers (pinned memory for an overlapped copy) must stay untouched until
 * dg_canvas_read_wait returns. Any later operation on this canvas is ordered
 * after the copy. */
dg_status dg_canvas_read_async(dg_ctx* ctx, int32_t canvas, uint8_t* bgra, float* depth);
/* Waits for the canvas's last dg_canvas_read_async; returns the error word of
 * the frames it waited for (without clearing it). */
dg_status dg_canvas_read_wait(dg_ctx* ctx, int32_t canvas);
dg_status dg_canvas_write(dg_ctx* ctx, int32_t canvas, const uint8_t* bgra, const float* depth);
/* Canvas::draw_triangle (canvas.rs:435-575), the GUI's 2D triangles, n of them
 * drawn in order: verts holds n x 3 vertices of 8 floats (x, y, u, v, r, g, b,
 * alpha; colour channels integers in 0..255, as Color::Custom), texmap the
 * texture map whose RGBA texels are blended (-1 = the 1x1 white default map),
 * clips NULL or n clipping rectangles (x_min, y_min, x_max, y_max). Each covered
 * pixel blends with the canvas where 0 < depth (the overlay does not write
 * depth). DG_E_INVALID for a clipping rectangle outside the canvas or a colour
 * out of range; DG_E_TEXTURE_RANGE as the reference's slice index panics. */
dg_status dg_canvas_draw_triangles_2d(dg_ctx* ctx, int32_t canvas, const float* verts, uint32_t n, int32_t texmap,
                                      const uint64_t* clips);
/* The frame as RGBA bytes (row 0 = top): bytes 0 and 2 of every pixel swapped
 * and the fourth kept, as Application::export_frame_as prepares it for
 * stbi_write_png/jpg (app/mod.rs:345-350). Synchronizes; returns kernel errors. */
dg_status dg_canvas_read_rgba(dg_ctx* ctx, int32_t canvas, uint8_t* rgba);
/* Device pointers of the canvas buffers (for zero-copy consumers). */
dg_status dg_canvas_device_ptrs(dg_ctx* ctx, int32_t canvas, void** bgra, void** depth);
dg_status dg_canvas_size(dg_ctx* ctx, int32_t canvas, uint64_t* width, uint64_t* height);

/* ------------------------------------------------------------------- render */
/* Scene::render(&mut canvas), scene/mod.rs:901-1249: enqueued on the context
 * stream; results are bit-identical to the reference's serial loop. */
dg_status dg_scene_render(dg_ctx* ctx, int32_t scene, int32_t canvas);
/* Renders n independent (scene, canvas) frames with one launch per pipeline
 * stage (the batched form). Equivalent to n dg_scene_render calls: a canvas
 * that appears again starts a new job, so the later frame overwrites it. */
dg_status dg_render_batch(dg_ctx* ctx, const int32_t* scenes, const int32_t* canvases, uint32_t n);

/* ---------------------------------------------------- graph-replayed batch
 * The batched form with its launch sequence captured in a CUDA graph: n
 * (scene, canvas) frames (scene/canvas ids of ctx) rendered as one job, like
 * dg_render_batch, but the descriptor upload, the counter reset and the
 * pipeline kernels are captured once and replayed by each dg_batch_render, so
 * a replay costs one graph launch on the context stream. Cameras, lights,
 * exponent, clear depth and canvas offsets may change between replays (the
 * host rewrites the uploaded descriptors); a change of shape (objects added to
 * a scene, a canvas resized or destroyed, texture maps added, dg_ctx_set_tuning)
 * is detected and re-captured at the next dg_batch_render. Each replay renders
 * exactly what n dg_scene_render calls would. The n canvases must be distinct
 * (DG_E_INVALID otherwise). The batch holds its own scratch memory; kernel
 * errors surface at the context's next synchronizing call. */
typedef struct dg_batch dg_batch;
dg_status dg_batch_create(dg_ctx* ctx, const int32_t* scenes, const int32_t* canvases, uint32_t n, dg_batch** out);
dg_status dg_batch_render(dg_batch* b);
/* [0] frames, [1] graph captures, [2] replays, [3] kernels per replay, [4] descriptor bytes per replay. */
dg_status dg_batch_info(dg_batch* b, uint64_t* out, int32_t n);
dg_status dg_batch_destroy(dg_batch* b);

/* Launch-shape autotuner: coordinate descent over the dg_tuning knobs on the
 * caller's frames (two sweeps; each candidate timed with CUDA events over
 * `reps` renders of the n frames after one warm-up render). Sets the fastest
 * tuning on ctx and returns it with its time per render in best_ms (either
 * pointer may be NULL). The knobs do not change what is rendered. The n
 * canvases must be distinct (DG_E_INVALID otherwise). */
dg_status dg_autotune(dg_ctx* ctx, const int32_t* scenes, const int32_t* canvases, uint32_t n, uint32_t reps,
                      dg_tuning* best, float* best_ms);

/* ------------------------------------------------------------ render server
 * Serving form of the draw call. The reference renders one frame per call of
 * Scene::render from its application loop (app/mod.rs:196); this server accepts
 * render requests from any thread as they arrive, keeps meshes and textures
 * resident (objects of the context), admits requests in arrival order against
 * a device-memory budget (each request holds W*H*16 bytes of colour, depth and
 * visibility buffers and 4 bytes per 32x32 pixel cell; job scratch counts too),
 * packs up to max_batch admitted requests into one batched render job, and
 * keeps up to `streams` jobs in flight on separate streams. With two or more
 * streams, requests of at least 1920x1080 pixels or 1M triangles wait in a
 * lane of their own, served by one stream in three (at least one) in batches
 * of at most 16, so smaller requests never queue behind them (a stream whose
 * lane has nothing pending takes the other lane's requests). Request buffers
 * are pooled per frame size and reused without a clear; pooled buffers count
 * against the budget and are released when a request of another size needs
 * the room. Each request renders exactly as dg_scene_render would render it
 * alone. While a server runs, its context must not be modified or used for
 * other rendering. */
typedef struct dg_server dg_server;

typedef struct {
    int32_t object;             /* object id from dg_object_create (opaque meshes only) */
    uint32_t width, height;     /* frame size: Scene::new(width, height) and its canvas */
    float cam_pos[3];
    float cam_dir[3];
    float near_, far_, fov_x_deg;
    float lights[DG_MAX_LIGHTS][3];
    uint32_t nlights;
    int32_t exponent;
    float clear_depth;          /* Canvas::init_depth value */
    int32_t discard;            /* 1: free the frame at completion (only status and latency are kept) */
} dg_request;

dg_status dg_server_create(dg_ctx* ctx, uint64_t budget_bytes, uint32_t max_batch, uint32_t streams,
                           dg_server** out);
/* Thread-safe. DG_E_OOM if the request alone exceeds the budget. */
dg_status dg_server_submit(dg_server* s, const dg_request* r, uint64_t* ticket);
/* Blocks until the request is done; copies its frame (BGRA, row 0 = top) and
 * depth to host memory when the pointers are not NULL, releases it, and
 * returns its status. latency_ms = completion - submission. */
dg_status dg_server_wait(dg_server* s, uint64_t ticket, uint8_t* bgra, float* depth, double* latency_ms);
/* [0] completed requests, [1] p50 latency ms, [2] p99 ms, [3] max ms, [4] batches,
 * [5] mean requests per batch, [6] peak device bytes held, [7] first launch error,
 * [8] request buffer sets allocated (the others were reused from the pool). */
dg_status dg_server_stats(dg_server* s, double* out, int32_t n);
/* Cancels a request that has not been admitted yet: it completes with
 * DG_E_CANCELLED (collect it with dg_server_wait). DG_E_INVALID when the ticket
 * is unknown or the request already runs or is done. */
dg_status dg_server_cancel(dg_server* s, uint64_t ticket);
/* Host-side fault injection for tests: the buffer allocation of this pending
 * request is made to fail as if the device were out of memory, so it completes
 * with DG_E_OOM while the rest of its batch renders. No GPU fault is involved.
 * DG_E_INVALID when the ticket is unknown or no longer pending. */
dg_status dg_server_inject_alloc_failure(dg_server* s, uint64_t ticket);
dg_status dg_server_reset_stats(dg_server* s);
/* Drains the pending requests, then frees the server. */
dg_status dg_server_destroy(dg_server* s);

/* ----------------------------------------------------- render without allocating
 * No counterpart in the reference: an extra entry point for callers that cannot
 * allocate device memory while they draw, for example a host application or
 * plugin that owns a fixed device-memory budget and hands the renderer only its
 * buffers, or a frame loop that must not stall on cudaMalloc/cudaFree (which
 * synchronize the device). It renders one frame of one mesh like
 * dg_scene_render, but all of its scratch memory (vertex records, the
 * visibility buffer, the raster queue, counters, the job descriptor) lives in
 * one statically sized __device__ array of the library (about 21 MiB, sized by
 * the limits below), which every GPU that loads the library keeps until the
 * process exits. It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * The caller passes its inputs and outputs as device pointers. Limits (checked,
 * DG_E_LIMIT beyond them): DG_NOALLOC_MAX_VERTICES position vertices,
 * DG_NOALLOC_MAX_TRIANGLES triangles, DG_NOALLOC_MAX_PIXELS canvas pixels,
 * DG_NOALLOC_MAX_LIGHTS lights, DG_NOALLOC_MAX_TEXMAPS texture maps,
 * DG_NOALLOC_MAX_MATERIALS materials. Precondition: every index is in range
 * (what dg_object_create validates for the allocating path); the indices stay
 * in device memory and are not read back.
 *
 * The work runs on the calling thread's current device, on `stream` (NULL = the
 * default stream). The first call on a device looks up the scratch array's
 * device address (cudaGetSymbolAddress) and keeps it for the life of the
 * process; make that first call before any stream capture, and do not call the
 * entry point across a cudaDeviceReset of that device (the kept address would
 * be stale). The call's job descriptor travels as a kernel parameter, so no
 * host buffer has to outlive the call. All calls share the one scratch array,
 * which keeps the last call's contents (each call re-initializes what must
 * start empty): calls whose GPU work overlaps, on different streams or host
 * threads, race and must not be issued. If status_out is not NULL the call
 * waits for its work and stores the first device-side error there: DG_OK,
 * DG_E_TEXTURE_RANGE (a texel offset past its map), or DG_E_CUDA (an internal
 * inconsistency, such as a material index beyond the materials passed). */
#define DG_NOALLOC_MAX_VERTICES 32768u
#define DG_NOALLOC_MAX_TRIANGLES 65536u
#define DG_NOALLOC_MAX_PIXELS 262144u
#define DG_NOALLOC_MAX_LIGHTS 2u
#define DG_NOALLOC_MAX_TEXMAPS 8u
#define DG_NOALLOC_MAX_MATERIALS 16u

/* A mesh resident in device memory, in the layout the kernels read:
 * pos float4[nv] (x, y, z, 1), nrm float4[nn] (x, y, z, 0), uv float2[nuv],
 * tri_pos uint4[ntri] (position indices a, b, c, material index),
 * tri_uv uint4[ntri] and tri_nrm uint4[ntri] (index triples, 4th word unused). */
typedef struct {
    const void* pos;
    const void* nrm;
    const void* uv;
    const void* tri_pos;
    const void* tri_uv;
    const void* tri_nrm;
    uint32_t nv, nn, nuv, ntri;
} dg_device_mesh;

/* A texture map in device memory: `len` image bytes (TextureMap layout, row 0 =
 * top), 4-byte aligned and readable up to the next multiple of 4 bytes plus 4. */
typedef struct {
    const void* bytes;
    uint64_t len;
    uint32_t width, height, components;
} dg_device_texmap;

/* Frame parameters: scene size (projection), canvas size, camera
 * (Camera::new(pos, dir, width/height) with explicit near/far/fov_x), lights,
 * specular exponent, depth clear value (Canvas::init_depth) and canvas offset. */
typedef struct {
    uint32_t width, height;
    uint32_t canvas_width, canvas_height;
    float cam_pos[3];
    float cam_dir[3];
    float near_, far_, fov_x_deg;
    float lights[DG_NOALLOC_MAX_LIGHTS][3];
    uint32_t nlights;
    int32_t exponent;
    float clear_depth;
    int32_t offset_x, offset_y;
} dg_frame_params;

/* Renders `mesh` with `materials` (map ids index `texmaps`, -1 = 1x1 white) into
 * bgra_out (u32[canvas pixels], Canvas byte layout) and depth_out
 * (f32[canvas pixels]), both device pointers. */
dg_status dg_render_noalloc(const dg_frame_params* params, const dg_device_mesh* mesh, const dg_material* materials,
                            uint32_t nmat, const dg_device_texmap* texmaps, uint32_t ntex, void* bgra_out,
                            void* depth_out, void* stream, int32_t* status_out);

#ifdef __cplusplus
}
#endif
#endif
