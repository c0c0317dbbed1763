/*
 * sgl.h — C ABI of the GB300 renderer for swegl scenes.
 *
 * The library keeps scenes resident in device memory and renders them with
 * hand-written sm_103a kernels.  Every entry point returns an sgl_status
 * (0 = success, negative = error); the text of the last error of a context is
 * available from sgl_last_error().  No entry point aborts or traps.
 *
 * Reference interfaces this ABI replaces (paths inside gbizzotto/swegl):
 *   swegl::render(scene_t&, T&... viewports)      swegl/render/renderer.hpp:27-34
 *   swegl::_render(scene_t&, viewport_t&)         src/render/renderer.cpp:77-235
 *   scene_t / node_t / primitive_t / mesh_vertex_t  swegl/data/model.hpp:20-178
 *   material_t / point_source_light               swegl/data/model.hpp:74-87
 *   texture_t / mipmap_t                          swegl/data/texture.hpp:12-38
 *   viewport_t(x, y, w, h, surface, shader, layers) swegl/render/viewport.hpp:27-62
 *   camera_t (view / projection matrices, centre) swegl/projection/camera.hpp:10-24
 *   pixel_shader_light_and_texture<pixel_shader_lights_phong,
 *       pixel_shader_texture_bilinear>            swegl/render/pixel_shaders.hpp:121-179
 *   post_shader_t::shade(viewport_t&)             swegl/render/post_shaders.hpp:33-47
 */
#ifndef SGL_H
#define SGL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SGL_API __attribute__((visibility("default")))
#else
#define SGL_API
#endif

typedef int sgl_status;

enum {
    SGL_OK              = 0,
    SGL_ERR_INVALID     = -1,  /* bad argument (null pointer, bad size, bad index)      */
    SGL_ERR_OOM         = -2,  /* device or host allocation failed                      */
    SGL_ERR_CUDA        = -3,  /* a CUDA runtime call failed                            */
    SGL_ERR_NOT_FOUND   = -4,  /* unknown scene id / ticket                             */
    SGL_ERR_BUDGET      = -5,  /* request can never fit the serving memory budget       */
    SGL_ERR_TIMEOUT     = -6,  /* a bounded wait ran out                                */
    SGL_ERR_NO_DEVICE   = -7,  /* no CUDA device                                        */
    SGL_ERR_UNSUPPORTED = -8,  /* feature the GPU path does not implement               */
    SGL_ERR_BUSY        = -9   /* result not ready yet (polling)                        */
};

/* primitive_t::index_mode_t (swegl/data/model.hpp:33-42); only the triangle
 * modes are rasterised by the reference. */
enum {
    SGL_TRIANGLES      = 4,
    SGL_TRIANGLE_STRIP = 5,
    SGL_TRIANGLE_FAN   = 6
};

/* ---------------------------------------------------------------- scenes -- */

/* node_t (swegl/data/model.hpp:50-71): local matrix = scale(rotation, scale)
 * followed by translate(translation); world = parent_world * local. */
typedef struct sgl_node_desc {
    float scale[3];
    float rotation[16];   /* row-major 4x4, matrix44_t layout */
    float translation[3];
    int   parent;         /* index of the parent node, -1 for a root node */
} sgl_node_desc;

/* primitive_t (swegl/data/model.hpp:31-48).  Vertices are owned by the
 * primitive: indices are local to [vertex_offset, vertex_offset+vertex_count),
 * and the vertex ranges of two primitives do not overlap (SGL_ERR_INVALID). */
typedef struct sgl_primitive_desc {
    int      node;
    int      mode;          /* SGL_TRIANGLES / SGL_TRIANGLE_STRIP / SGL_TRIANGLE_FAN */
    int      material;      /* index into materials; -1 selects default_material */
    uint32_t vertex_offset;
    uint32_t vertex_count;
    uint32_t index_offset;
    uint32_t index_count;
} sgl_primitive_desc;

/* material_t (swegl/data/model.hpp:80-87).  `shininess` is the point-light
 * specular exponent; the reference hard-codes 32 (src/render/pixel_shaders.cpp:192). */
typedef struct sgl_material_desc {
    uint32_t color;         /* 0xAARRGGBB, used when texture == -1 */
    int      texture;       /* index into textures, -1 = none */
    int      double_sided;
    int      shininess;     /* integer exponent, 1..1024 */
} sgl_material_desc;

/* texture_t mip level 0 (swegl/data/texture.hpp:12-27): 0xAARRGGBB texels. */
typedef struct sgl_texture_desc {
    const uint32_t *texels;
    int             width;
    int             height;
} sgl_texture_desc;

/* point_source_light (swegl/data/model.hpp:74-78) */
typedef struct sgl_point_light {
    float position[3];
    float intensity;
} sgl_point_light;

/* scene_t (swegl/data/model.hpp:128-178), flattened: vertex attributes are
 * structure-of-arrays (positions xyz, normals xyz, uvs uv). */
typedef struct sgl_scene_desc {
    int                        n_nodes;
    const sgl_node_desc       *nodes;
    int                        n_primitives;
    const sgl_primitive_desc  *primitives;
    uint32_t                   n_vertices;
    const float               *positions;   /* 3 * n_vertices */
    const float               *normals;     /* 3 * n_vertices */
    const float               *uvs;         /* 2 * n_vertices */
    uint32_t                   n_indices;
    const uint32_t            *indices;
    int                        n_materials;
    const sgl_material_desc   *materials;
    int                        n_textures;
    const sgl_texture_desc    *textures;
    int                        n_point_lights;
    const sgl_point_light     *point_lights;
    float                      ambient;          /* scene_t::ambient_light_intensity */
    float                      sun_direction[3]; /* scene_t::sun_direction (normalised) */
    float                      sun_intensity;    /* scene_t::sun_intensity */
    sgl_material_desc          default_material; /* scene_t::default_material */
} sgl_scene_desc;

/* ----------------------------------------------------------------- views -- */

/* Depth-of-field gather (replaces post_shader_depth_box,
 * swegl/render/post_shaders.hpp:51-132, whose own output is not usable).  It
 * runs over the view's rectangle after the view is rendered; for a view with
 * transparency layers, after the layers are flattened and copied to the
 * surface (the reference's post shader reads the first layer), with the
 * view's opaque depth. */
typedef struct sgl_dof_desc {
    int   enabled;
    float focus;        /* view-space focus distance */
    float aperture;     /* lens aperture in world units */
    float max_radius;   /* circle of confusion clamp, pixels (0..4096) */
    float px_scale;     /* pixels per world unit at unit distance; 0 = P11*h/2 */
} sgl_dof_desc;

/* The viewport's pixel shader (viewport_t::m_pixel_shader, a
 * pixel_shader_t of swegl/render/pixel_shaders.hpp).  The combinations are
 * pixel_shader_light_and_texture<L, T> (pixel_shaders.hpp:121-179); the
 * single shaders write what their shade() returns (for the light shaders,
 * the light value 65536 * L as the int colour, as the reference does). */
enum {
    SGL_SHADER_PHONG_BILINEAR = 0, /* <pixel_shader_lights_phong, pixel_shader_texture_bilinear> */
    SGL_SHADER_PHONG_NEAREST  = 1, /* <pixel_shader_lights_phong, pixel_shader_texture> */
    SGL_SHADER_FLAT_BILINEAR  = 2, /* <pixel_shader_lights_flat, pixel_shader_texture_bilinear> */
    SGL_SHADER_FLAT_NEAREST   = 3, /* <pixel_shader_lights_flat, pixel_shader_texture> */
    SGL_SHADER_COLOR          = 4, /* pixel_shader_t: the material colour */
    SGL_SHADER_BILINEAR       = 5, /* pixel_shader_texture_bilinear */
    SGL_SHADER_NEAREST        = 6, /* pixel_shader_texture */
    SGL_SHADER_PHONG          = 7, /* pixel_shader_lights_phong */
    SGL_SHADER_FLAT           = 8, /* pixel_shader_lights_flat */
    SGL_SHADER_COUNT          = 9
};

/* viewport_t + camera_t (swegl/render/viewport.hpp:27-62,
 * swegl/projection/camera.hpp:10-24). */
typedef struct sgl_view {
    int          x, y, w, h;        /* viewport rectangle inside the target surface */
    float        view[16];          /* camera_t::m_viewmatrix, row-major */
    float        proj[16];          /* camera_t::m_projectionmatrix, row-major */
    float        camera_pos[3];     /* camera_t::m_center */
    sgl_dof_desc dof;
    int          shader;            /* SGL_SHADER_*; 0 = Phong + bilinear */
    int          layers;            /* transparency layers (viewport_t's transparency_layer_count),
                                       0 = opaque; 1..SGL_MAX_LAYERS (not in debug, autotune or
                                       allocation-free renders) */
} sgl_view;

#define SGL_MAX_LAYERS 8

/* The SDL_Surface fields the reference writes (pixels, pitch, w, h with
 * BytesPerPixel = 4) plus viewport_t::m_zbuffer (w*h floats of the view). */
typedef struct sgl_target {
    void  *pixels;      /* BGRA8 surface */
    int    pitch;       /* bytes per surface row */
    int    width;       /* surface width in pixels */
    int    height;      /* surface height in pixels */
    float *zbuffer;     /* view w*h depth values, may be NULL */
} sgl_target;

/* Per-frame counters filled by sgl_render when `stats` is non-NULL. */
typedef struct sgl_frame_stats {
    uint64_t triangles;       /* triangles in the scene */
    uint64_t drawn_triangles; /* (sub-)triangles that reached scanline setup */
    uint64_t fragments;       /* covered (triangle, pixel) pairs of all spans */
    uint64_t pixels;          /* viewport pixels written */
    uint32_t kernel_launches; /* kernels this call launched */
    uint32_t reserved;
} sgl_frame_stats;

/* ----------------------------------------------------------- entry points -- */

typedef struct sgl_ctx sgl_ctx;

/* Create a context on CUDA `device`.  One context per host thread, or
 * external locking: a context is not re-entrant. */
SGL_API sgl_status sgl_create(sgl_ctx **out, int device);
SGL_API void       sgl_destroy(sgl_ctx *ctx);
SGL_API const char *sgl_last_error(const sgl_ctx *ctx);
SGL_API const char *sgl_status_string(sgl_status status);
SGL_API int        sgl_version(void);

/* Copy a scene into device memory (replaces the per-frame scene_t walk of
 * renderer.cpp:83-231).  Host arrays may be freed after the call. */
SGL_API sgl_status sgl_scene_upload(sgl_ctx *ctx, const sgl_scene_desc *desc, int *scene_id);
SGL_API sgl_status sgl_scene_release(sgl_ctx *ctx, int scene_id);
/* Replace node transforms (scene_t::animate, model.hpp:146-177). */
SGL_API sgl_status sgl_scene_set_nodes(sgl_ctx *ctx, int scene_id, const sgl_node_desc *nodes, int n_nodes);
/* Replace the lights (scene_t ambient / sun / point_source_lights). */
SGL_API sgl_status sgl_scene_set_lights(sgl_ctx *ctx, int scene_id, float ambient,
                                        const float sun_direction[3], float sun_intensity,
                                        const sgl_point_light *lights, int n_lights);
SGL_API sgl_status sgl_scene_info(sgl_ctx *ctx, int scene_id, uint64_t *n_triangles, uint64_t *n_vertices,
                                  uint64_t *device_bytes);

/* swegl::render(scene, vp...) (renderer.hpp:27-34) for the
 * Phong + bilinear shader: world transform once, then each view in order.
 * `targets[i]` receives view i.  When `device_buffers` is 0 the target
 * pointers are host memory and the call copies in and out (synchronous);
 * when 1 they are device memory and the call is asynchronous on `stream`
 * (a cudaStream_t, NULL = legacy default stream). */
SGL_API sgl_status sgl_render(sgl_ctx *ctx, int scene_id, const sgl_view *views, const sgl_target *targets,
                              int n_views, int device_buffers, void *stream, sgl_frame_stats *stats);

/* sgl_render for one view, for callers that must not allocate: a real-time
 * frame callback with a fixed memory plan, or a host that forbids the library
 * from growing its footprint or from taking the device-wide synchronisation
 * of cudaMalloc / cudaFree.  No counterpart in the reference (its render call
 * allocates nothing on a GPU because it has none).  All scratch comes from one
 * 64 MiB static device array that every GPU loading the library keeps until
 * exit; views needing more are refused with SGL_ERR_BUDGET.  Targets are
 * device buffers; asynchronous on `stream`.  The array is shared by every
 * call in a CUDA context (each context has its own copy): calls that overlap
 * on the GPU in one context race, so order them.  The first call in a context
 * looks up the array's address there (cudaGetSymbolAddress) and caches it
 * under the context's id; make that first call before any stream capture. */
SGL_API sgl_status sgl_render_noalloc(sgl_ctx *ctx, int scene_id, const sgl_view *view, const sgl_target *target,
                                      void *stream);

/* Debug variant of one view: writes the per-pixel winner slot
 * (2 * draw-order triangle index + clip sub-triangle, 0xFFFFFFFF = none) and
 * the per-slot "reached scanline setup" flags, used to check depth-test
 * winners bit-exactly.  Host buffers; `winner` holds w*h, `slot_flags`
 * 2 * n_triangles bytes. */
SGL_API sgl_status sgl_render_debug(sgl_ctx *ctx, int scene_id, const sgl_view *view, const sgl_target *target,
                                    uint32_t *winner, uint8_t *slot_flags, sgl_frame_stats *stats);

/* ------------------------------------------------------------- batching -- */

/* Batched renderer: many views, of one or several resident scenes and of
 * uneven sizes, rendered by one launch sequence (one CUDA graph launch when
 * use_graph is set).  Targets are device buffers and must not overlap.
 * Replaces a loop of swegl::_render calls (src/render/renderer.cpp:77-235)
 * over independent viewports. */
typedef struct sgl_batch_opts {
    int tile;      /* shade tile edge: 8, 16 or 32 pixels (0 = context default) */
    int span_bin;  /* spans wider than this many pixels are binned to the
                      warp-cooperative span kernels (1..64, 0 = default 16) */
    int use_graph; /* run the launch sequence as a captured CUDA graph */
} sgl_batch_opts;

typedef struct sgl_batch_item {
    int        scene_id;
    sgl_view   view;
    sgl_target target; /* device buffers */
    /* Optional pose of this item alone: the scene's n_nodes node transforms
     * to render it with (e.g. from sgl_gltf_animate at the item's time); NULL
     * renders the scene's current nodes.  Many poses of one resident scene
     * render in one batch; the scene's own nodes are untouched. */
    const sgl_node_desc *nodes;
    int        n_nodes;
} sgl_batch_item;

/* Asynchronous on `stream` unless `stats` is requested (then it waits).
 * Items with transparency layers run after the others, each as its own
 * launch sequence in item order, and the call waits for them. */
SGL_API sgl_status sgl_render_batch(sgl_ctx *ctx, const sgl_batch_item *items, int n_items,
                                    const sgl_batch_opts *opts, void *stream, sgl_frame_stats *stats);
/* Times every tile x span_bin choice on this batch and returns the fastest. */
SGL_API sgl_status sgl_autotune(sgl_ctx *ctx, const sgl_batch_item *items, int n_items, sgl_batch_opts *chosen);

/* ------------------------------------------------------- depth of field -- */

/* The depth-of-field gather alone on a rendered view (replaces
 * post_shader_t::shade / post_shader_depth_box::shade,
 * swegl/render/post_shaders.hpp:33-132, whose own output is not usable: it
 * reads a z-buffer the opaque path never writes).  `in` holds the view's
 * colour rectangle and z-buffer, `out` receives the gathered colour in its
 * rectangle.  Per pixel: view depth z = (z' - P23) / P22 from the z-buffer,
 * circle of confusion r = K * aperture * |z - focus| / z pixels (K =
 * px_scale, or P11 * h / 2 when 0) clamped to [0, max_radius], and the mean of
 * the 32 taps of sgl_dof_taps.h at offsets r * tap rounded to the nearest
 * integer (ties to even) and clamped to the
 * view, integer sums rounded half up; alpha is kept.  sgl_render applies the
 * same gather to every view whose dof.enabled is set. */
SGL_API sgl_status sgl_dof(sgl_ctx *ctx, const sgl_view *view, const sgl_target *in, const sgl_target *out,
                           int device_buffers, void *stream);

/* -------------------------------------------------------------- serving -- */

/* A request loop that keeps scenes resident, admits render requests of any
 * scene and viewport size against a device-memory budget (framebuffer +
 * scratch bytes), batches them as they arrive and keeps several batches in
 * flight on separate streams (continuous batching).  No reference
 * counterpart: the reference renders one frame per call of
 * swegl::render (src/test_1.cpp:365-376). */
typedef struct sgl_server sgl_server;

typedef struct sgl_serve_opts {
    uint64_t budget_bytes; /* device bytes admitted at once (0 = 40 GiB) */
    int      max_batch;    /* views per batch (0 = 64) */
    int      streams;      /* batches in flight (0 = 3) */
    int      copy_out;     /* 1 = copy each frame to the request's host buffers */
} sgl_serve_opts;

typedef struct sgl_request {
    int       scene_id;
    sgl_view  view;          /* x, y ignored: the frame is w x h */
    uint32_t *host_pixels;   /* w*h BGRA8, written when copy_out (may be NULL) */
    float    *host_zbuffer;  /* w*h depth, written when copy_out (may be NULL) */
    /* Optional pose of this request alone (animated serving): the scene's
     * n_nodes node transforms to render with, e.g. from sgl_gltf_animate at
     * the request's time; NULL renders the scene's current nodes.  Copied at
     * submit. */
    const sgl_node_desc *nodes;
    int       n_nodes;
} sgl_request;

typedef struct sgl_request_result {
    sgl_status status;
    double     submit_s, start_s, done_s; /* steady host clock, seconds; done_s: delivered (after the copy to
                                             the host buffers when the server copies out) */
    double     rendered_s;                /* when the frame was complete in device memory: done_s less the
                                             device time of the batch's copies to the host (= done_s
                                             without copy-out) */
    uint64_t   fragments;                 /* covered (triangle, pixel) pairs */
} sgl_request_result;

SGL_API sgl_status sgl_server_create(sgl_ctx *ctx, const sgl_serve_opts *opts, sgl_server **out);
/* Queue a request; SGL_ERR_BUDGET when it alone exceeds the budget. */
SGL_API sgl_status sgl_server_submit(sgl_server *srv, const sgl_request *req, uint64_t *ticket);
/* Queue n requests in one call (each as sgl_server_submit would; a host
 * binding through a foreign-function interface pays its call overhead once
 * instead of per request).  tickets[i] receives request i's ticket; stops
 * at the first request that is refused and returns its status, with
 * *n_queued (may be NULL) the number queued before it.  No reference
 * counterpart (the reference has no serving loop). */
SGL_API sgl_status sgl_server_submit_batch(sgl_server *srv, const sgl_request *reqs, int n, uint64_t *tickets,
                                           int *n_queued);
/* SGL_OK with the result (once per ticket), SGL_ERR_BUSY while in flight. */
SGL_API sgl_status sgl_server_poll(sgl_server *srv, uint64_t ticket, sgl_request_result *result);
SGL_API sgl_status sgl_server_wait(sgl_server *srv, uint64_t ticket, double timeout_s, sgl_request_result *result);
/* Wait for n tickets; results[i] (may be NULL) receives ticket i's result.
 * SGL_ERR_TIMEOUT when they are not all done within timeout_s (the results
 * of the tickets before the one waited for are filled and consumed). */
SGL_API sgl_status sgl_server_wait_batch(sgl_server *srv, const uint64_t *tickets, int n, double timeout_s,
                                         sgl_request_result *results);
/* Wait until every submitted request is done (SGL_ERR_TIMEOUT otherwise). */
SGL_API sgl_status sgl_server_drain(sgl_server *srv, double timeout_s);
/* Batches and kernels launched, requests completed so far. */
SGL_API sgl_status sgl_server_stats(sgl_server *srv, uint64_t *batches, uint64_t *kernels, uint64_t *completed);
SGL_API void       sgl_server_destroy(sgl_server *srv);

/* Page-locked host memory for request frames (cudaHostAlloc on the current
 * device; `write_combined` adds cudaHostAllocWriteCombined).  Frames copied
 * into write-combined memory kept their delivery rate on GB300 hosts where
 * copies into ordinary page-locked memory slowed down the longer the host ran
 * (27.6-28.1 k against 19.9-29.8 k frames/s end to end); CPU reads of it
 * measured the same as of ordinary memory there.  Free with sgl_host_free.
 * No reference counterpart (the reference renders into host surfaces). */
SGL_API sgl_status sgl_host_alloc(size_t bytes, int write_combined, void **out);
SGL_API sgl_status sgl_host_free(void *p);

/* Device-side bounds checks.  The library built with them (libsgl_check.so,
 * compiled with -DSGL_BOUNDS_CHECK beside libsgl.so) tests the index of each
 * guarded device access — projected vertices, set-up records, depth keys,
 * winner records, output pixels, texels — against its buffer; an index outside
 * is recorded (the first failure's check code and index, and a count) and the
 * access skipped, so nothing traps.  Reads the record (and clears it when
 * `reset`); SGL_ERR_UNSUPPORTED from the library without the checks.  No
 * reference counterpart (a stand-in for a memory checker). */
SGL_API sgl_status sgl_check_status(sgl_ctx *ctx, uint32_t *code, uint64_t *index, uint32_t *count, int reset);

/* Per-kernel device timing (CUDA events on the launching stream around each
 * kernel of every frame rendered while enabled).  Enabling resets the totals.
 * Kernels are numbered 0..n-1; reading past the last returns SGL_ERR_NOT_FOUND.
 * No reference counterpart: the reference's only timer is the demo's frame
 * clock (src/test_1.cpp:365-376). */
SGL_API sgl_status sgl_profile(sgl_ctx *ctx, int enable);
SGL_API sgl_status sgl_profile_read(sgl_ctx *ctx, int kernel, const char **name, double *total_ms,
                                    uint64_t *launches);

/* ------------------------------------------------------------ glTF scenes -- */

/* swegl::load_scene (src/data/gltf.cpp:388-464): a .gltf file (JSON whose
 * buffers and images are files next to it, or base64 data URIs) or a .glb
 * file read into host memory as a scene description, with the reference
 * loader's rules (see the notes of swegl_gb300/csrc/sgl_gltf.cpp): images
 * decoded (BMP, PNG, baseline JPEG; src/misc/image.cpp:20-265), animations kept for
 * sgl_gltf_animate.  Host only: no context or device is needed.  On failure
 * `error` (if given) receives a message. */
typedef struct sgl_gltf sgl_gltf;
SGL_API sgl_status sgl_gltf_load(const char *path, sgl_gltf **out, char *error, size_t error_size);
/* The scene description, valid until sgl_gltf_free; its nodes follow the
 * animations.  Like a loaded scene_t it has no lights (ambient, sun and
 * point lights zero): set them on a copy before sgl_scene_upload. */
SGL_API const sgl_scene_desc *sgl_gltf_scene(const sgl_gltf *g);
SGL_API int                   sgl_gltf_animation_count(const sgl_gltf *g);
/* scene_t::animate(seconds) (swegl/data/model.hpp:146-177): every animation
 * at `seconds` modulo its length, keyframes interpolated linearly, rotations
 * normalised; the nodes' scale, rotation and translation are updated and,
 * if `nodes` is given, all sgl_gltf_scene()->n_nodes of them written there
 * for sgl_scene_set_nodes. */
SGL_API sgl_status sgl_gltf_animate(sgl_gltf *g, float seconds, sgl_node_desc *nodes);
SGL_API void       sgl_gltf_free(sgl_gltf *g);

/* read_image_file (src/misc/image.cpp:20-27): a BMP, PNG or baseline JPEG
 * file (chosen by its extension) decoded to 0xAARRGGBB texels, row 0 first;
 * free them with sgl_image_free. */
SGL_API sgl_status sgl_image_load(const char *path, uint32_t **texels, int *width, int *height, char *error,
                                  size_t error_size);
SGL_API void       sgl_image_free(uint32_t *texels);

#ifdef __cplusplus
}
#endif

#endif /* SGL_H */
