/* A plain C client of include/rle_gb300.h, as a reference-side integration
 * would be written: no C++, no Python.  Built and run by tests/test_c_abi.py.
 *
 *   abi_client host    scene generation, .rle4 round trip through the
 *                      loader's validation, ray maps, error paths (no GPU)
 *   abi_client gpu     additionally renders one frame on device 0 through
 *                      rle_render_frame and checks it is not empty
 * Exit status 0 on success; every failure prints the call and status. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rle_gb300.h"

#define CHECK(call)                                                                                  \
    do {                                                                                             \
        rle_status st_ = (call);                                                                     \
        if (st_ != RLE_OK) {                                                                         \
            fprintf(stderr, "%s:%d %s -> %s (%s)\n", __FILE__, __LINE__, #call, rle_status_string(st_), \
                    rle_last_error());                                                               \
            return 1;                                                                                \
        }                                                                                            \
    } while (0)

#define EXPECT(cond)                                                                 \
    do {                                                                             \
        if (!(cond)) {                                                               \
            fprintf(stderr, "%s:%d expected %s\n", __FILE__, __LINE__, #cond);       \
            return 1;                                                                \
        }                                                                            \
    } while (0)

/* the CUDA runtime's allocation calls, declared here so this file needs no
 * CUDA headers (the library links the runtime statically; the GPU mode is
 * linked against libcudart as well) */
extern int cudaMalloc(void** p, size_t n);
extern int cudaFree(void* p);
extern int cudaMemcpy(void* dst, const void* src, size_t n, int kind);
extern int cudaDeviceSynchronize(void);

static int host_checks(void** bytes_out, size_t* n_out) {
    printf("%s\n", rle_version());
    rle_scenegen_params p;
    CHECK(rle_scenegen_default(128, 128, 128, 9, 1, &p));
    EXPECT(p.nummaps == 4 && p.sx == 128);
    void* bytes = NULL;
    size_t n = 0;
    CHECK(rle_scenegen_rle4(&p, &bytes, &n));
    EXPECT(bytes != NULL && n > 16);
    /* the .rle4 header: level count, then per level sx, sy, sz, words */
    int32_t head[5];
    memcpy(head, bytes, sizeof(head));
    EXPECT(head[0] == 4 && head[1] == 128 && head[2] == 128 && head[3] == 128);

    rle_camera cam = {{64.5f, -100.0f, 64.5f}, {0.2f, 1.0f, 0.0f}, 90.0f};
    rle_view_params v = {640, 480, 0, 0, 0.0f, 0, 0};
    rle_raymap rm;
    CHECK(rle_raymap_build(&cam, &v, &rm));
    EXPECT(rm.samples == 640 && rm.rays > 0 && rm.rays <= rm.rows);
    EXPECT(rle_raybuf_words(&rm) == (size_t)rm.rows * (size_t)rm.samples);
    EXPECT(rle_frame_workspace_bytes(&v) > 0);

    /* refused inputs come back as status codes */
    rle_view_params tall = {100, 200, 0, 0, 0.0f, 0, 0};
    EXPECT(rle_raymap_build(&cam, &tall, &rm) == RLE_ERR_INVALID_ARG);
    rle_camera bad = cam;
    bad.pos[0] = NAN;
    EXPECT(rle_raymap_build(&bad, &v, &rm) == RLE_ERR_INVALID_ARG);
    rle_scene* s = NULL;
    EXPECT(rle_scene_load_memory(bytes, 6, 0, &s) == RLE_ERR_FORMAT && s == NULL);
    EXPECT(rle_scene_load_file("/nonexistent/scene.rle4", 0, &s) == RLE_ERR_IO);
    EXPECT(strcmp(rle_status_string(RLE_ERR_CAPACITY), "RLE_ERR_CAPACITY") == 0);
    *bytes_out = bytes;
    *n_out = n;
    return 0;
}

static int gpu_checks(const void* bytes, size_t n) {
    rle_scene* s = NULL;
    CHECK(rle_scene_load_memory(bytes, n, 0, &s));
    rle_scene_info info;
    CHECK(rle_scene_get_info(s, &info));
    EXPECT(info.nummaps == 4 && info.sx[0] == 128 && info.run_headers > 0);
    rle_camera cam = {{64.5f, -120.0f, 64.5f}, {0.3f, 0.7f, 0.0f}, 90.0f};
    rle_view_params v = {320, 240, 0, 0, 0.0f, 64, 0};
    const size_t ws_bytes = rle_frame_workspace_bytes(&v);
    void *ws = NULL, *colour = NULL, *depth = NULL;
    EXPECT(cudaMalloc(&ws, ws_bytes) == 0);
    EXPECT(cudaMalloc(&colour, 320 * 240 * 4) == 0);
    EXPECT(cudaMalloc(&depth, 320 * 240 * 4) == 0);
    CHECK(rle_render_frame(s, &cam, &v, ws, ws_bytes, (uint32_t*)colour, (float*)depth, NULL, NULL));
    EXPECT(cudaDeviceSynchronize() == 0);
    uint32_t* host = (uint32_t*)malloc(320 * 240 * 4);
    EXPECT(cudaMemcpy(host, colour, 320 * 240 * 4, 2 /* device to host */) == 0);
    int sky = 0, ground = 0;
    for (int i = 0; i < 320 * 240; i++) {
        if (host[i] == 0xffffccb2u) sky++;
        else if (host[i] != 0) ground++;
    }
    printf("sky %d, terrain %d pixels\n", sky, ground);
    EXPECT(ground > 1000);
    free(host);
    cudaFree(ws);
    cudaFree(colour);
    cudaFree(depth);
    CHECK(rle_scene_free(s));
    return 0;
}

int main(int argc, char** argv) {
    const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
    void* bytes = NULL;
    size_t n = 0;
    if (host_checks(&bytes, &n)) return 1;
    if (gpu && gpu_checks(bytes, n)) return 1;
    rle_host_free(bytes);
    printf("ok\n");
    return 0;
}
