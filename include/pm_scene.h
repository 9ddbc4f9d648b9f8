/*
 * pm_scene.h -- seeded synthetic equirectangular scenes with analytic ground
 * truth, for tests and benchmarks of the densifier.
 *
 * The reference ships no posed stereo data for its dense path (its demo video
 * and dataset are not distributed with the source), so every workload here is
 * generated: a camera inside a textured box room, optionally with axis-aligned
 * boxes and a vertical cylinder, or a long hall of boxes for trajectories.
 * Surfaces carry a solid (3-D) value-noise texture of 4 octaves mapped to
 * 0..255, so the same surface point has the same intensity in every view.
 *
 * Conventions match the densifier: pixel (i, j) has bearing
 * (cos(lat) sin(lon), -sin(lat), cos(lat) cos(lon)) with lon = 2 pi (j/W - 1/2)
 * and lat = -pi (i/H - 1/2); poses are world->camera (R_cw row-major, t_cw);
 * depth is the range along the bearing (metres).
 */
#ifndef PM_SCENE_H
#define PM_SCENE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pm_scene pm_scene;

enum {
    PM_SCENE_ROOM = 0,          /* 10 x 6 x 3 m room */
    PM_SCENE_ROOM_OBJECTS = 1,  /* room + 5 boxes (0.3-1.5 m) + 1 cylinder (r = 0.5 m) */
    PM_SCENE_HALL = 2           /* 30 x 10 x 4 m hall of textured boxes */
};

/* Create a scene of the given kind; the layout and texture derive from seed. */
pm_scene *pm_scene_create(int kind, uint32_t seed);
void pm_scene_destroy(pm_scene *s);

/* Poses of one request: view 0 is the reference camera (free space, random
 * yaw); views 1..n_views-1 are offset from it by a baseline uniform in
 * [bmin, bmax] metres in a uniform random 3-D direction, with a random yaw of
 * +-yaw_deg degrees relative to the reference.  R: n_views*9, t: n_views*3.
 * Returns 0 on success. */
int pm_scene_poses(const pm_scene *s, int n_views, uint32_t seed, float bmin, float bmax,
                   float yaw_deg, double *R, double *t);

/* Camera pose on the scene's seeded smooth trajectory (Catmull-Rom spline
 * through n_waypoints random free-space waypoints, traversed over
 * duration_s seconds) at time t_s, with a slowly varying yaw. */
int pm_scene_trajectory_pose(const pm_scene *s, uint32_t seed, int n_waypoints, double duration_s,
                             double t_s, double R[9], double t[3]);

/* Render one view.  Any output may be NULL.
 *   gray   : H*W float intensities (0..255; integer-valued unless noise_sigma > 0)
 *   gray_u8: H*W bytes (rounded, clamped)
 *   rgb    : H*W*3 bytes, BGR order (like the reference's rgb thumbnails)
 *   depth  : H*W float range along the bearing
 *   normal : H*W*3 float unit surface normal in the camera frame (facing the camera)
 * supersample: s*s sub-samples averaged per pixel (1 = point sampling).
 * noise_sigma > 0 adds seeded Gaussian noise (0..255 scale) to gray. */
int pm_scene_render(const pm_scene *s, const double R[9], const double t[3], int W, int H,
                    int supersample, float noise_sigma, uint32_t noise_seed, float *gray,
                    uint8_t *gray_u8, uint8_t *rgb, float *depth, float *normal);

/* Plain description of a scene (for the device renderer). */
#define PM_SCENE_MAX_BOXES 32
#define PM_SCENE_MAX_CYLS 4
typedef struct {
    double room_lo[3], room_hi[3];
    int n_boxes, n_cyls;
    double box_lo[PM_SCENE_MAX_BOXES][3], box_hi[PM_SCENE_MAX_BOXES][3];
    double cyl[PM_SCENE_MAX_CYLS][5]; /* cx, cz, r, y0, y1 */
    uint32_t seed;
    double base_freq;
} pm_scene_desc;
int pm_scene_describe(const pm_scene *s, pm_scene_desc *out);

/* Render one view on the GPU into caller-owned device buffers (any may be
 * NULL): gray_u8 H*W, depth H*W (range), bgr H*W*3.  Same scene, texture and
 * conventions as pm_scene_render, evaluated in FP32; noise_sigma > 0 adds
 * hashed Gaussian noise.  Enqueued on `stream` (a cudaStream_t). */
int pm_scene_render_device(const pm_scene *s, const double R[9], const double t[3], int W, int H, int supersample,
                           float noise_sigma, uint32_t noise_seed, uint8_t *gray_u8, float *depth, uint8_t *bgr,
                           void *stream);

/* The unrounded intensities (0..255 scale, noise added) of the device
 * renderer as H*W floats, for FP16 image studies. */
int pm_scene_render_device_f32(const pm_scene *s, const double R[9], const double t[3], int W, int H,
                               int supersample, float noise_sigma, uint32_t noise_seed, float *gray, void *stream);

#ifdef __cplusplus
}
#endif
#endif
