/*
 * fauxglcuda.h -- C ABI of libfauxglcuda, the GB300 (sm_103a) implementation of
 * FauxGL's triangle pipeline.
 *
 * The ABI is what a cgo wrapper of package fauxgl binds: plain C types,
 * opaque handles, host arrays borrowed only for the duration of a call. Every function returns an fgc_status (0 = FGC_OK). A failing call
 * leaves a message retrievable with fgc_last_error().
 *
 * Reference interfaces replaced (file:line in fogleman/fauxgl):
 *   fgc_context_create      NewContext                     context.go:60-81
 *   fgc_clear_color         Context.ClearColorBufferWith   context.go:119-131
 *                           (ClearColorBuffer = ...With(dc.ClearColor), context.go:133-135)
 *   fgc_clear_depth         Context.ClearDepthBufferWith   context.go:137-141
 *                           (ClearDepthBuffer = ...With(math.MaxFloat64), context.go:143-145)
 *   fgc_mesh_upload         Mesh{Triangles, Lines}         mesh.go:9-13 (+ Triangle/Line/Vertex,
 *                                                          triangle.go:3-5, line.go:3-5, vertex.go:3-12)
 *   fgc_texture_upload      ImageTexture                   texture.go:21-31
 *   fgc_draw_mesh           Context.DrawMesh               context.go:435-439
 *   fgc_draw_triangles      Context.DrawTriangles          context.go:413-433
 *                           (DrawTriangle = a draw of one triangle, context.go:370-389)
 *   fgc_draw_lines          Context.DrawLines              context.go:391-411
 *                           (DrawLine = a draw of one line, context.go:351-368)
 *   fgc_read_color          Context.Image / ColorBuffer    context.go:83-85, 43
 *   fgc_read_depth          Context.DepthBuffer            context.go:44
 *   fgc_write_color/_depth  host writes into ColorBuffer / DepthBuffer (public fields)
 *   fgc_depth_image         Context.DepthImage             context.go:87-117
 *   fgc_downsample          (no reference counterpart: the examples call the third-party
 *                           resize.Resize after Image(), README.md:107-109)
 *   fgc_mesh_load_stl       LoadSTL                        stl.go:23-154 (+ Triangle.Normal,
 *                                                          triangle.go:33-37)
 *   fgc_mesh_smooth_normals_threshold  Mesh.SmoothNormalsThreshold  mesh.go:80-103
 *   fgc_mesh_smooth_normals            Mesh.SmoothNormals           mesh.go:105-120
 *   fgc_mesh_sharp_edges               Mesh.SharpEdges              mesh.go:258-292
 *   fgc_mesh_silhouette                Mesh.Silhouette              mesh.go:207-209,
 *                                                                   silhouette.go:3-53
 *   fgc_mesh_download       the Triangles / Lines of a Mesh (mesh.go:9-13), read back
 *
 * Draw state (fgc_state) mirrors the public Context fields (context.go:40-58);
 * shader parameters (fgc_shader) mirror SolidColorShader / TextureShader /
 * PhongShader (shader.go:10-59). A Go Shader that is not one of the three
 * built-ins cannot be expressed here: the wrapper rejects it with an error,
 * there is no CPU fallback.
 */
#ifndef FAUXGLCUDA_H
#define FAUXGLCUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FGC_ABI_VERSION 3

typedef enum fgc_status {
    FGC_OK = 0,
    FGC_ERR_INVALID_ARGUMENT = 1,   /* bad handle, size or enum value              */
    FGC_ERR_UNSUPPORTED_SHADER = 2, /* shader kind is not a built-in               */
    FGC_ERR_CUDA = 3,               /* a CUDA runtime call failed                  */
    FGC_ERR_OUT_OF_MEMORY = 4,      /* device allocation failed                    */
    FGC_ERR_DEVICE_LIMIT = 5,       /* a kernel hit a bounded limit and gave up     */
    FGC_ERR_UNSUPPORTED = 6,        /* valid request outside what this build does  */
    FGC_ERR_BUSY = 7                /* the context has draws in an unfinished batch */
} fgc_status;

/* Face and Cull take the reference's enum values (context.go:11-26). */
enum { FGC_FACE_CW = 1, FGC_FACE_CCW = 2 };
enum { FGC_CULL_NONE = 1, FGC_CULL_FRONT = 2, FGC_CULL_BACK = 3 };

/* Built-in shader kinds (shader.go). */
enum { FGC_SHADER_SOLID_COLOR = 1, FGC_SHADER_TEXTURE = 2, FGC_SHADER_PHONG = 3 };

/* Arithmetic forms. PLAIN computes every stage in FP64 in the reference's
 * operation order. MIXED keeps FP64 for the vertex transform, triangle setup,
 * edge functions and depth, and runs interpolation and shading in FP32. */
enum { FGC_PRECISION_PLAIN = 0, FGC_PRECISION_MIXED = 1 };

/* Debug outputs a context may keep beside its framebuffer (fgc_context_set_debug). */
enum { FGC_DEBUG_WINNER = 1, FGC_DEBUG_SHADED_COLOR = 2 };

typedef struct fgc_context fgc_context;
typedef struct fgc_mesh fgc_mesh;
typedef struct fgc_texture fgc_texture;

/* RasterizeInfo (context.go:28-31). */
typedef struct fgc_rasterize_info {
    uint64_t total_pixels;
    uint64_t updated_pixels;
} fgc_rasterize_info;

/* Per-draw snapshot of the public Context fields (context.go:40-58). Booleans
 * are 0/1. NewContext's defaults (context.go:66-77) are what
 * fgc_state_default() writes. */
typedef struct fgc_state {
    int32_t read_depth;
    int32_t write_depth;
    int32_t write_color;
    int32_t alpha_blend;
    int32_t wireframe;
    int32_t front_face;   /* FGC_FACE_*                    */
    int32_t cull;         /* FGC_CULL_*                    */
    int32_t precision;    /* FGC_PRECISION_* (new knob)    */
    double line_width;
    double depth_bias;
} fgc_state;

/* Built-in shader parameters (shader.go:10-59). matrix is row-major
 * (Matrix.X00, X01, ... X33, matrix.go:5-10). color is SolidColorShader.Color
 * or PhongShader.ObjectColor. texture is TextureShader.Texture or
 * PhongShader.Texture (NULL = none). */
typedef struct fgc_shader {
    int32_t kind;         /* FGC_SHADER_* */
    int32_t reserved;
    double matrix[16];
    double color[4];
    double light_direction[3];
    double camera_position[3];
    double ambient_color[4];
    double diffuse_color[4];
    double specular_color[4];
    double specular_power;
    const fgc_texture* texture;
} fgc_shader;

/* ---- library ------------------------------------------------------------ */
int32_t fgc_abi_version(void);
/* Fill *st with NewContext's defaults (context.go:66-77): ReadDepth, WriteDepth,
 * WriteColor, AlphaBlend on; Wireframe off; FaceCCW; CullBack; LineWidth 2;
 * DepthBias 0; precision PLAIN. */
void fgc_state_default(fgc_state* st);
/* NewSolidColorShader / NewTextureShader / NewPhongShader (shader.go:14-16, 33-35, 61-68). */
void fgc_shader_solid_color(fgc_shader* sh, const double matrix[16], const double rgba[4]);
void fgc_shader_texture(fgc_shader* sh, const double matrix[16], const fgc_texture* tex);
void fgc_shader_phong(fgc_shader* sh, const double matrix[16], const double light_direction[3],
                      const double camera_position[3]);
/* Message of the last failed call on this thread (never NULL). */
const char* fgc_last_error(void);

/* ---- context ------------------------------------------------------------ */
/* NewContext(width, height): device-resident NRGBA colour (4 B/px) and FP64
 * depth (8 B/px) buffers. The colour buffer starts transparent (all zero) and
 * the depth buffer at math.MaxFloat64, as in the reference. Uses the current
 * CUDA device; every call on the context runs on the context's own stream. */
int fgc_context_create(int32_t width, int32_t height, fgc_context** out);
int fgc_context_destroy(fgc_context* ctx);
int fgc_context_size(const fgc_context* ctx, int32_t* width, int32_t* height);
/* Keep winner ids (element index of the last fragment that updated each pixel,
 * lines with bit 31 set, 0xFFFFFFFF where none) and/or the FP64 shader output
 * of that fragment, for parity tests. 0 turns both off. */
int fgc_context_set_debug(fgc_context* ctx, int32_t flags);

/* ClearColorBufferWith(c): every pixel becomes c.NRGBA() (color.go:56-63). */
int fgc_clear_color(fgc_context* ctx, const double rgba[4]);
/* ClearDepthBufferWith(v). */
int fgc_clear_depth(fgc_context* ctx, double value);

/* ---- resources ---------------------------------------------------------- */
/* Upload a triangle soup plus a line list as a device-resident mesh.
 *   tri_pos  ntri*9   V1.Position xyz, V2.Position xyz, V3.Position xyz
 *   tri_nrm  ntri*9   normals, same layout, or NULL (all zero)
 *   tri_tex  ntri*6   Vertex.Texture X,Y per corner, or NULL (Texture.Z never
 *                     reaches an output and is not stored)
 *   tri_col  ntri*12  Vertex.Color RGBA per corner, or NULL
 *   line_*   the same per line with 2 corners (6, 6, 4, 8 values per line).
 * Host arrays are read during the call only. The mesh lives on the current
 * device and may be drawn by any context on that device. */
int fgc_mesh_upload(const double* tri_pos, const double* tri_nrm, const double* tri_tex,
                    const double* tri_col, uint64_t ntri,
                    const double* line_pos, const double* line_nrm, const double* line_tex,
                    const double* line_col, uint64_t nline, fgc_mesh** out);
int fgc_mesh_release(fgc_mesh* mesh);
int fgc_mesh_counts(const fgc_mesh* mesh, uint64_t* ntri, uint64_t* nline);

/* Mesh preparation on the device. Positions, normals and the position
 * grouping of the reference's map[Vector] (== on float64: -0 and +0 are one
 * key, a NaN position is never found) are computed with the reference's
 * FP64 operation order, so results are the reference's bits; SharpEdges
 * compares CUDA's acos with the threshold, which may decide differently from
 * Go's math.Acos for an angle within an ulp or two of it.
 *
 * fgc_mesh_load_stl: the bytes of an STL file. Binary when its size is
 * 84 + 50 * (the header's triangle count), else ASCII ("vertex x y z" lines,
 * three per triangle). Positions are the file's (FP32 widened to FP64 for
 * binary); every corner's normal is the triangle's Normal().
 * fgc_mesh_smooth_normals_threshold / _smooth_normals replace the triangle
 * corners' normals in place (call with no draw of the mesh in flight).
 * fgc_mesh_sharp_edges / fgc_mesh_silhouette create a line mesh (release it
 * with fgc_mesh_release); the input is not changed.
 * fgc_mesh_download copies positions and normals (3 doubles per corner) into
 * any non-null array: tri_* 9 per triangle, line_* 6 per line. */
int fgc_mesh_load_stl(const void* data, uint64_t nbytes, fgc_mesh** out);
int fgc_mesh_smooth_normals_threshold(fgc_mesh* mesh, double radians);
int fgc_mesh_smooth_normals(fgc_mesh* mesh);
int fgc_mesh_sharp_edges(const fgc_mesh* mesh, double angle_threshold, fgc_mesh** out);
int fgc_mesh_silhouette(const fgc_mesh* mesh, const double eye[3], double offset, fgc_mesh** out);
int fgc_mesh_download(const fgc_mesh* mesh, double* tri_pos, double* tri_nrm, double* line_pos, double* line_nrm);

/* ImageTexture: texels as the 16-bit alpha-premultiplied RGBA that
 * image.Image.At(x, y).RGBA() returns, row-major, width*height*4 values.
 * BilinearSample (texture.go:41-63) converts them with MakeColor (color.go:25-29). */
int fgc_texture_upload(const uint16_t* rgba16, int32_t width, int32_t height, fgc_texture** out);
int fgc_texture_release(fgc_texture* tex);

/* ---- drawing ------------------------------------------------------------ */
/* DrawMesh: all triangles, then all lines, in submission order; fragments
 * resolve per pixel exactly as the reference's sequential DrawTriangle /
 * DrawLine loop would. *info receives the summed RasterizeInfo. Blocks until
 * the draw has finished. */
int fgc_draw_mesh(fgc_context* ctx, const fgc_mesh* mesh, const fgc_state* st,
                  const fgc_shader* sh, fgc_rasterize_info* info);
/* DrawTriangles over mesh triangles [first, first+count). */
int fgc_draw_triangles(fgc_context* ctx, const fgc_mesh* mesh, uint64_t first, uint64_t count,
                       const fgc_state* st, const fgc_shader* sh, fgc_rasterize_info* info);
/* DrawLines over mesh lines [first, first+count). */
int fgc_draw_lines(fgc_context* ctx, const fgc_mesh* mesh, uint64_t first, uint64_t count,
                   const fgc_state* st, const fgc_shader* sh, fgc_rasterize_info* info);

/* ---- buffers ------------------------------------------------------------ */
/* Copy the NRGBA colour buffer (width*height*4 bytes, rows top to bottom). */
int fgc_read_color(fgc_context* ctx, uint8_t* nrgba);
/* Copy the FP64 depth buffer (width*height values). */
int fgc_read_depth(fgc_context* ctx, double* depth);
/* Replace the colour / depth buffer from host memory. */
int fgc_write_color(fgc_context* ctx, const uint8_t* nrgba);
int fgc_write_depth(fgc_context* ctx, const double* depth);
/* DepthImage (context.go:87-117): Gray16 normalisation of the depth buffer
 * (width*height uint16 values). */
int fgc_depth_image(fgc_context* ctx, uint16_t* gray16);
/* DepthImage without any device allocation (no counterpart in the
 * reference). fgc_depth_image allocates its device staging buffers the first
 * time it runs; a caller that must not have the library allocate GPU memory
 * after start-up -- a render service that sizes every buffer before it admits
 * requests, or a host application that owns the device memory of the plugins
 * it loads -- calls this instead. The scratch is one static 16 MiB device
 * array, reserved on a GPU (together with the kernels this call launches)
 * when the first context on that GPU is created, and held until the process
 * exits; frames are limited to FGC_DEPTH_IMAGE_NOALLOC_MAX_PIXELS pixels and
 * larger contexts get FGC_ERR_INVALID_ARGUMENT. All calls share the array:
 * calls that overlap on the GPU race. */
#define FGC_DEPTH_IMAGE_NOALLOC_MAX_PIXELS 8388608
int fgc_depth_image_noalloc(fgc_context* ctx, uint16_t* gray16);
/* Box-downsample the colour buffer by an integer factor on the device:
 * out is (width/scale)*(height/scale)*4 bytes; each output channel is the
 * rounded mean (sum + n/2) / n of the scale*scale input bytes. width and
 * height must be multiples of scale. */
int fgc_downsample(fgc_context* ctx, int32_t scale, uint8_t* out);
/* Debug outputs (see fgc_context_set_debug). */
int fgc_read_winner(fgc_context* ctx, uint32_t* winner);
int fgc_read_shaded_color(fgc_context* ctx, double* rgba);

/* ---- instrumentation (no reference counterpart) ------------------------- */
/* Work counters and stage times of the context's last draw. Stage times are
 * filled only while timing is on (fgc_context_set_timing): CUDA events
 * recorded on the draw's stream between the pipeline stages. */
enum { FGC_STAGE_VERTEX = 0, FGC_STAGE_SETUP = 1, FGC_STAGE_CLIP = 2, FGC_STAGE_BIN = 3,
       FGC_STAGE_RASTER = 4, FGC_STAGE_COUNT = 5 };
typedef struct fgc_stats {
    uint64_t elements;          /* triangles + lines submitted                     */
    uint64_t unique_vertices;   /* vertex-stage invocations (welded positions)     */
    uint64_t clipped;           /* elements that went through clipping             */
    uint64_t primitives;        /* raster primitive slots                          */
    uint64_t bin_entries;       /* (primitive, band) pairs                         */
    uint64_t visited_pixels;    /* pixels stepped by the edge walk                 */
    uint64_t covered_pixels;    /* in-frame covered pixels (TotalPixels)           */
    uint64_t shaded_fragments;  /* fragments shaded (after early depth rejection)  */
    uint64_t updated_pixels;    /* UpdatedPixels                                   */
    uint64_t kernel_launches;   /* kernels launched by the draw (all attempts)     */
    uint32_t bands, band_rows, attempts, reserved;
    double stage_ms[FGC_STAGE_COUNT];
} fgc_stats;
int fgc_context_set_timing(fgc_context* ctx, int32_t enable);
int fgc_context_last_stats(const fgc_context* ctx, fgc_stats* out);
/* Run the context's work on a caller-owned cudaStream_t (NULL restores the
 * context's own stream). */
int fgc_context_set_stream(fgc_context* ctx, void* cuda_stream);
/* Test hook for the failure path of the draw pipeline's bounded waits (no
 * reference counterpart). The binning stage's scans (bin offsets, row-start
 * slots) run in one pass by a decoupled look-back in which each block waits,
 * a bounded number of polls, for its predecessors to publish their sums; a
 * wait that runs out makes the draw return FGC_ERR_DEVICE_LIMIT with its
 * framebuffers untouched. spin_limit sets that number of polls (0: the default,
 * 2^22) and withhold_block names a logical block that never publishes
 * (0xFFFFFFFF: none), so a test can make the waits run out on purpose; the
 * setting is process-wide and applies to draws issued after the call. */
int fgc_debug_lookback(uint32_t spin_limit, uint32_t withhold_block);
/* FP64 pipe throughput of the current device, measured: independent FP64
 * adds issued on every SM, in G instructions per second. It is the roofline
 * denominator of the FP64-bound stages, whose arithmetic is adds and
 * multiplies (both issue at this rate; a fused multiply-add of general
 * operands issues about 1.19x faster). */
int fgc_measure_fp64_rate(double* gops_per_s);

/* ---- batches (no reference counterpart) --------------------------------- */
/* A batch renders many independent draws -- views of uneven size, each with
 * its own mesh range, state, shader and target context -- with one launch per
 * pipeline stage for all of them: a persistent raster launch walks the
 * (draw, band) queue of the whole batch. Every draw's output, RasterizeInfo
 * included, is exactly what fgc_draw_triangles / fgc_draw_lines on its own
 * would give. Draws run in list order; draws that share a context, or that
 * differ in precision, go to successive passes of the same submission.
 *
 * fgc_batch_submit returns once the work is queued on the batch's stream;
 * fgc_batch_wait blocks until it is done (re-running a pass whose buffers
 * overflowed) and fills one fgc_rasterize_info per draw. Between the two, the
 * contexts of the draws are busy: any other call on them returns
 * FGC_ERR_BUSY. A draw with out_nrgba set has its frame copied there after
 * the batch, box-downsampled by out_scale (1 = the frame itself; out_scale
 * must divide the frame): (width/out_scale)*(height/out_scale)*4 bytes, best
 * in page-locked memory. One submission is in flight per batch; use several
 * batches (each with its own stream) to overlap submissions. */
typedef struct fgc_batch fgc_batch;
typedef struct fgc_batch_item {
    fgc_context* context;
    const fgc_mesh* mesh;
    uint64_t tri_first, tri_count;    /* triangles [first, first+count)   */
    uint64_t line_first, line_count;  /* then lines [first, first+count)  */
    const fgc_state* state;
    const fgc_shader* shader;
    uint8_t* out_nrgba;               /* optional read-back destination    */
    int32_t out_scale;                /* 0 or 1: no downsampling           */
    int32_t reserved;
} fgc_batch_item;
/* Shapes of the batched pipeline. Results never depend on them;
 * fgc_batch_autotune picks them by measurement. */
typedef struct fgc_batch_tuning {
    int32_t band_pixels;          /* raster band size in pixels, whole rows (default 4096) */
    int32_t prims_per_bin_block;  /* primitives per binning block (default 4096)           */
    int32_t fragment_cap;         /* fragment buffer of a raster CTA (default 1024)        */
    int32_t use_graph;            /* 1: issue each submission as a CUDA graph              */
    int32_t window;               /* raster pixels per thread and round for wide triangles (default 8) */
    int32_t reserved;
} fgc_batch_tuning;
int fgc_batch_create(fgc_batch** out);
int fgc_batch_destroy(fgc_batch* b);
int fgc_batch_set_stream(fgc_batch* b, void* cuda_stream);
int fgc_batch_set_tuning(fgc_batch* b, const fgc_batch_tuning* t);
int fgc_batch_get_tuning(const fgc_batch* b, fgc_batch_tuning* t);
int fgc_batch_set_timing(fgc_batch* b, int32_t enable);
int fgc_batch_submit(fgc_batch* b, const fgc_batch_item* items, uint64_t n);
/* *done = 1 once the submitted work has finished on the device (no wait). */
int fgc_batch_query(fgc_batch* b, int32_t* done);
int fgc_batch_wait(fgc_batch* b, fgc_rasterize_info* infos);
/* Counters (summed over the draws) and stage times of the last finished submission. */
int fgc_batch_last_stats(const fgc_batch* b, fgc_stats* out);
/* Render items `repeats` times under each candidate tuning, keep the fastest
 * in the batch and write it to *best. The items' contexts are drawn into
 * (clear them before real use). */
int fgc_batch_autotune(fgc_batch* b, const fgc_batch_item* items, uint64_t n, int32_t repeats,
                       fgc_batch_tuning* best);

#ifdef __cplusplus
}
#endif

#endif /* FAUXGLCUDA_H */
