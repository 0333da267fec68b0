/* C11 program against include/rtbvh.h, linked to librtbvh_rs.so.
 *
 * Compile-time: the sizes and field offsets of every ABI struct, as the
 * reference's same_size test pins them (rtbvh_ffi/src/lib.rs:855-866:
 * RTBvhNode = BvhNode, RTMbvhNode = MbvhNode, RTAabb = Aabb).
 * Run time, mode "args" (no GPU needed): the argument errors of
 * create_delete (rtbvh_ffi/src/lib.rs:868-904) return before any device work.
 * Mode "gpu": create_delete and the intersect test (:945-1019) -- two
 * triangles forming the quad z = 1, a ray from the origin along +z through
 * both the Bvh and the Mbvh host-callback entry points must find t == 1. */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "rtbvh.h"

_Static_assert(sizeof(RTAabb) == 32, "RTAabb is 32 bytes");
_Static_assert(offsetof(RTAabb, min) == 0 && offsetof(RTAabb, count) == 12, "RTAabb min/count");
_Static_assert(offsetof(RTAabb, max) == 16 && offsetof(RTAabb, left_first) == 28, "RTAabb max/left_first");
_Static_assert(sizeof(RTBvhNode) == 32 && offsetof(RTBvhNode, aabb) == 0, "RTBvhNode is an RTAabb");
_Static_assert(sizeof(RTMbvhNode) == 128, "RTMbvhNode is 128 bytes");
_Static_assert(offsetof(RTMbvhNode, min_x) == 0 && offsetof(RTMbvhNode, max_x) == 16, "RTMbvhNode x");
_Static_assert(offsetof(RTMbvhNode, min_y) == 32 && offsetof(RTMbvhNode, max_y) == 48, "RTMbvhNode y");
_Static_assert(offsetof(RTMbvhNode, min_z) == 64 && offsetof(RTMbvhNode, max_z) == 80, "RTMbvhNode z");
_Static_assert(offsetof(RTMbvhNode, children) == 96 && offsetof(RTMbvhNode, counts) == 112, "RTMbvhNode ids");
_Static_assert(sizeof(RTBvh) == 32 && sizeof(RTMbvh) == 32, "handles are 32 bytes");
_Static_assert(offsetof(RTBvh, id) == 0 && offsetof(RTBvh, node_count) == 4 && offsetof(RTBvh, nodes) == 8,
               "RTBvh head");
_Static_assert(offsetof(RTBvh, index_count) == 16 && offsetof(RTBvh, indices) == 24, "RTBvh tail");
_Static_assert(offsetof(RTMbvh, nodes) == 8 && offsetof(RTMbvh, indices) == 24, "RTMbvh");
_Static_assert(sizeof(ResultCode) == 4 && sizeof(BvhType) == 4, "enums are 32-bit");
_Static_assert(Ok == 0 && Error == 1 && NoPrimitives == 2 && InequalAabbsAndPrimitives == 3 && Nan == 4,
               "ResultCode values");
_Static_assert(LocallyOrderedClustered == 0 && BinnedSAH == 1, "BvhType values");
/* this library's trace flags: distinct bits */
_Static_assert(RTBVH_TRACE_ANY_HIT == 1u && RTBVH_TRACE_STATS == 2u && RTBVH_TRACE_REORDER == 4u &&
                   RTBVH_TRACE_EXACT_NODES == 8u && RTBVH_TRACE_WALK_STATS == 16u,
               "trace flags");

static int failures = 0;
#define CHECK(cond)                                                  \
  do {                                                               \
    if (!(cond)) {                                                   \
      fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                    \
    }                                                                \
  } while (0)

typedef struct {
  float origin[3], direction[3];
  const float (*vertices)[3];
} UserData;

static void sub3(const float* a, const float* b, float* r) {
  r[0] = a[0] - b[0];
  r[1] = a[1] - b[1];
  r[2] = a[2] - b[2];
}
static void cross3(const float* a, const float* b, float* r) {
  r[0] = a[1] * b[2] - b[1] * a[2];
  r[1] = a[2] * b[0] - b[2] * a[0];
  r[2] = a[0] * b[1] - b[0] * a[1];
}
static float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* the test's own callback: Moller-Trumbore on triangle `id`, shrinking *t */
static bool intersect_test(uint32_t id, float* t, void* data) {
  const UserData* d = (const UserData*)data;
  const float *v0 = d->vertices[3 * id], *v1 = d->vertices[3 * id + 1], *v2 = d->vertices[3 * id + 2];
  float e1[3], e2[3], h[3], s[3], q[3];
  sub3(v1, v0, e1);
  sub3(v2, v0, e2);
  cross3(d->direction, e2, h);
  const float a = dot3(e1, h);
  if (a > -1e-5f && a < 1e-5f) return false;
  const float f = 1.0f / a;
  sub3(d->origin, v0, s);
  const float u = f * dot3(s, h);
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  cross3(s, e1, q);
  const float v = f * dot3(d->direction, q);
  if (v < 0.0f || u + v > 1.0f) return false;
  const float tv = f * dot3(e2, q);
  if (tv > 1e-5f && tv < *t) *t = tv;
  return false;
}

static void box_of(const float (*v)[3], RTAabb* b) {
  for (int k = 0; k < 3; ++k) {
    b->min[k] = fminf(fminf(v[0][k], v[1][k]), v[2][k]);
    b->max[k] = fmaxf(fmaxf(v[0][k], v[1][k]), v[2][k]);
  }
  b->count = 0;
  b->left_first = 0;
}

static void args_mode(void) {
  RTBvh bvh;
  memset(&bvh, 0, sizeof(bvh));
  /* create_delete: no centres -> Error (rtbvh_ffi/src/lib.rs:889-901) */
  CHECK(create_bvh(NULL, 27, NULL, 16, 1, BinnedSAH, &bvh) == Error);
  /* no result pointer -> Error */
  float centers[4 * 27] = {0};
  CHECK(create_bvh(NULL, 27, centers, 16, 1, BinnedSAH, NULL) == Error);
  /* a centre stride other than 12 or 16 (the reference aborts) -> Error */
  CHECK(create_bvh(NULL, 27, centers, 20, 1, BinnedSAH, &bvh) == Error);
  CHECK(create_mbvh(bvh, NULL) == Error);
  CHECK(rtbvh_gpu_version() != NULL);
}

static void gpu_mode(void) {
  /* create_delete (rtbvh_ffi/src/lib.rs:868-939): 27 triangles over a grid */
  float grid[100][3];
  for (int x = 0; x <= 9; ++x)
    for (int y = 0; y <= 9; ++y) {
      grid[x * 10 + y][0] = (float)x;
      grid[x * 10 + y][1] = (float)y;
      grid[x * 10 + y][2] = 0.0f;
    }
  RTAabb aabbs[27];
  float centers[27][4];
  for (int i = 0; i < 27; ++i) {
    box_of((const float(*)[3])grid[3 * i], &aabbs[i]);
    for (int k = 0; k < 3; ++k) centers[i][k] = (aabbs[i].min[k] + aabbs[i].max[k]) * 0.5f;
    centers[i][3] = 0.0f;
  }
  RTBvh bvh;
  RTMbvh mbvh;
  CHECK(create_bvh(NULL, 27, &centers[0][0], 16, 1, BinnedSAH, &bvh) == Ok);
  free_bvh(bvh);
  CHECK(create_bvh(aabbs, 27, &centers[0][0], 16, 1, BinnedSAH, &bvh) == Ok);
  CHECK(create_mbvh(bvh, &mbvh) == Ok);
  free_bvh(bvh);
  free_mbvh(mbvh);

  /* intersect (:945-1019): the quad z = 1 as two triangles, centres as vec3 (stride 12) */
  static const float quad[6][3] = {{-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};
  RTAabb qb[2];
  float qc[2][3];
  for (int i = 0; i < 2; ++i) {
    box_of(&quad[3 * i], &qb[i]);
    for (int k = 0; k < 3; ++k) qc[i][k] = (qb[i].min[k] + qb[i].max[k]) * 0.5f;
  }
  CHECK(create_bvh(qb, 2, &qc[0][0], 12, 1, BinnedSAH, &bvh) == Ok);
  CHECK(create_mbvh(bvh, &mbvh) == Ok);
  UserData ud = {{0, 0, 0}, {0, 0, 1}, quad};
  float t = 1e26f;
  CHECK(intersect(bvh, ud.origin, ud.direction, &t, &ud, intersect_test) == Ok);
  CHECK(fabsf(t - 1.0f) < 1.1920929e-7f);
  t = 1e26f;
  CHECK(intersect_mbvh(mbvh, ud.origin, ud.direction, &t, &ud, intersect_test) == Ok);
  CHECK(fabsf(t - 1.0f) < 1.1920929e-7f);
  /* the same quad through the GPU closest-hit entry point */
  free_bvh(bvh);
  free_mbvh(mbvh);
}

int main(int argc, char** argv) {
  if (argc > 1 && strcmp(argv[1], "gpu") == 0) gpu_mode();
  else args_mode();
  if (failures) {
    fprintf(stderr, "%d checks failed\n", failures);
    return 1;
  }
  printf("abi_check.c ok\n");
  return 0;
}
