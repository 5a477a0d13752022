/*
 * fauxgl_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of fogleman/fauxgl's triangle pipeline (context.go,
 * clipping.go, vertex.go, shader.go, texture.go, color.go, vector.go,
 * matrix.go, util.go), used as the checker for the GPU library and, in its
 * multi-threaded form, as the timed CPU baseline. Nothing in the product
 * (package fauxgl_gb300, libfauxglcuda) links or calls this code.
 *
 * Parity unpinned: the reference ships no tests, golden vectors or fixtures
 * for this path and its Go sources cannot be built here (no Go toolchain on
 * either machine). The restatement is pinned by hand-derived known-answer
 * tests (tests/test_oracle_kat.py) instead.
 *
 * Build with -ffp-contract=off: the reference's semantics are unfused IEEE
 * FP64 (Go on amd64 does not contract x*y+z).
 */
#ifndef FAUXGL_ORACLE_H
#define FAUXGL_ORACLE_H

#include <stdint.h>
#include "../include/fauxglcuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* NewContext (context.go:60-81). */
oracle_ctx* oracle_create(int32_t width, int32_t height);
void oracle_destroy(oracle_ctx* ctx);
void oracle_clear_color(oracle_ctx* ctx, const double rgba[4]);
void oracle_clear_depth(oracle_ctx* ctx, double value);

/* Mesh arrays: same layout as fgc_mesh_upload. texture: 16-bit premultiplied
 * RGBA texels (tex_w*tex_h*4) or NULL.
 * nthreads == 0: sequential DrawTriangle/DrawLine loop in submission order
 *                (the oracle; deterministic).
 * nthreads >= 1: the reference's own concurrency (context.go:391-433):
 *                nthreads workers, worker wi takes elements i with
 *                i % nthreads == wi, 256 striped locks keyed by (x+y)&255,
 *                unlocked early depth read. Used as the CPU baseline; its
 *                output is as non-deterministic as the reference's.
 * what: 1 = triangles only, 2 = lines only, 3 = both (DrawMesh). */
int oracle_draw(oracle_ctx* ctx, const fgc_state* st, const fgc_shader* sh,
                const uint16_t* texture, int32_t tex_w, int32_t tex_h,
                const double* tri_pos, const double* tri_nrm, const double* tri_tex,
                const double* tri_col, int64_t tri_first, int64_t tri_count,
                const double* line_pos, const double* line_nrm, const double* line_tex,
                const double* line_col, int64_t line_first, int64_t line_count,
                int32_t what, int32_t nthreads, fgc_rasterize_info* info);

uint8_t* oracle_color(oracle_ctx* ctx);      /* W*H*4 NRGBA            */
double* oracle_depth(oracle_ctx* ctx);       /* W*H                    */
uint32_t* oracle_winner(oracle_ctx* ctx);    /* W*H element ids        */
double* oracle_shaded(oracle_ctx* ctx);      /* W*H*4 FP64 shader out  */

/* Box downsample (the project's definition; parity unpinned). */
void oracle_downsample(const uint8_t* src, int32_t width, int32_t height, int32_t scale,
                       uint8_t* dst);
/* DepthImage (context.go:87-117). */
void oracle_depth_image(oracle_ctx* ctx, uint16_t* gray16);

/* Exposed helpers for known-answer tests. */
double oracle_go_pow(double x, double y);
void oracle_nrgba(const double c[4], uint8_t out[4]);
void oracle_blend(uint8_t dst[4], const double src[4]);
int oracle_clip_triangle(const double clip[12], double out_clip[7 * 3 * 4]);

/* Mesh preparation (fauxgl_oracle_mesh.c): stl.go, mesh.go:80-120, 258-292,
 * silhouette.go. Lines are 6 doubles (two points); counts beyond cap are
 * returned but not written. */
int64_t oracle_stl_parse(const uint8_t* data, uint64_t n, double* tri_pos, double* tri_nrm, uint64_t cap);
void oracle_smooth_normals_threshold(const double* tri_pos, double* tri_nrm, uint64_t ntri, double threshold);
void oracle_smooth_normals(const double* tri_pos, double* tri_nrm, uint64_t ntri);
int64_t oracle_sharp_edges(const double* tri_pos, uint64_t ntri, double angle_threshold, double* out, uint64_t cap);
int64_t oracle_silhouette(const double* tri_pos, const double* tri_nrm, uint64_t ntri, const double eye[3],
                          double offset, double* out, uint64_t cap);

#ifdef __cplusplus
}
#endif

#endif
