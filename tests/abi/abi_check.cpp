// C++17 program against include/rtbvh.hpp (namespace rtbvh, enum class
// types, the reference's cbindgen C++ form), linked to librtbvh_rs.so.
// Same checks as abi_check.c: struct sizes and offsets
// (rtbvh_ffi/src/lib.rs:855-866) at compile time; in mode "args" the
// argument errors of create_delete (:868-904); in mode "gpu" create_delete
// and the t == 1 quad of the intersect test (:945-1019) through the Bvh and
// Mbvh host-callback entry points.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "rtbvh.hpp"

using rtbvh::BvhType;
using rtbvh::ResultCode;
using rtbvh::RTAabb;
using rtbvh::RTBvh;
using rtbvh::RTBvhNode;
using rtbvh::RTMbvh;
using rtbvh::RTMbvhNode;

static_assert(sizeof(RTAabb) == 32 && offsetof(RTAabb, count) == 12 && offsetof(RTAabb, max) == 16 &&
                  offsetof(RTAabb, left_first) == 28,
              "RTAabb layout");
static_assert(sizeof(RTBvhNode) == 32, "RTBvhNode is an RTAabb");
static_assert(sizeof(RTMbvhNode) == 128 && offsetof(RTMbvhNode, max_x) == 16 && offsetof(RTMbvhNode, min_y) == 32 &&
                  offsetof(RTMbvhNode, max_z) == 80 && offsetof(RTMbvhNode, children) == 96 &&
                  offsetof(RTMbvhNode, counts) == 112,
              "RTMbvhNode layout");
static_assert(sizeof(RTBvh) == 32 && offsetof(RTBvh, nodes) == 8 && offsetof(RTBvh, index_count) == 16 &&
                  offsetof(RTBvh, indices) == 24,
              "RTBvh layout");
static_assert(sizeof(RTMbvh) == 32 && offsetof(RTMbvh, indices) == 24, "RTMbvh layout");
static_assert(std::is_same<std::underlying_type<BvhType>::type, uint32_t>::value, "BvhType is repr(u32)");
static_assert(sizeof(ResultCode) == 4, "ResultCode is a C enum");
static_assert(static_cast<int>(ResultCode::Nan) == 4 && static_cast<uint32_t>(BvhType::BinnedSAH) == 1, "values");
static_assert(std::is_standard_layout<RTAabb>::value && std::is_trivially_copyable<RTMbvhNode>::value, "POD");
static_assert(RTBVH_TRACE_ANY_HIT == 1u && RTBVH_TRACE_STATS == 2u && RTBVH_TRACE_REORDER == 4u &&
                  RTBVH_TRACE_EXACT_NODES == 8u && RTBVH_TRACE_WALK_STATS == 16u,
              "trace flags, the same bits as rtbvh.h");

static int failures = 0;
#define CHECK(cond)                                                               \
  do {                                                                            \
    if (!(cond)) {                                                                \
      std::fprintf(stderr, "%s:%d: check failed: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                                 \
    }                                                                             \
  } while (0)

namespace {

struct Vec3 {
  float x, y, z;
};
Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
Vec3 cross(Vec3 a, Vec3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float dot(Vec3 a, Vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

struct UserData {
  Vec3 origin, direction;
  const Vec3* vertices;
};

bool intersect_test(uint32_t id, float* t, void* data) {
  const UserData& d = *static_cast<const UserData*>(data);
  const Vec3 v0 = d.vertices[3 * id], v1 = d.vertices[3 * id + 1], v2 = d.vertices[3 * id + 2];
  const Vec3 e1 = v1 - v0, e2 = v2 - v0, h = cross(d.direction, e2);
  const float a = dot(e1, h);
  if (a > -1e-5f && a < 1e-5f) return false;
  const float f = 1.0f / a;
  const Vec3 s = d.origin - v0;
  const float u = f * dot(s, h);
  if (!(u >= 0.0f && u <= 1.0f)) return false;
  const Vec3 q = cross(s, e1);
  const float v = f * dot(d.direction, q);
  if (v < 0.0f || u + v > 1.0f) return false;
  const float tv = f * dot(e2, q);
  if (tv > 1e-5f && tv < *t) *t = tv;
  return false;
}

RTAabb box_of(const Vec3* v) {
  RTAabb b{};
  b.min[0] = std::fmin(std::fmin(v[0].x, v[1].x), v[2].x);
  b.min[1] = std::fmin(std::fmin(v[0].y, v[1].y), v[2].y);
  b.min[2] = std::fmin(std::fmin(v[0].z, v[1].z), v[2].z);
  b.max[0] = std::fmax(std::fmax(v[0].x, v[1].x), v[2].x);
  b.max[1] = std::fmax(std::fmax(v[0].y, v[1].y), v[2].y);
  b.max[2] = std::fmax(std::fmax(v[0].z, v[1].z), v[2].z);
  return b;
}

void args_mode() {
  RTBvh bvh{};
  CHECK(rtbvh::create_bvh(nullptr, 27, nullptr, 16, 1, BvhType::BinnedSAH, &bvh) == ResultCode::Error);
  float centers[4 * 27] = {};
  CHECK(rtbvh::create_bvh(nullptr, 27, centers, 16, 1, BvhType::BinnedSAH, nullptr) == ResultCode::Error);
  CHECK(rtbvh::create_bvh(nullptr, 27, centers, 20, 1, BvhType::BinnedSAH, &bvh) == ResultCode::Error);
  CHECK(rtbvh::create_mbvh(bvh, nullptr) == ResultCode::Error);
  CHECK(rtbvh::rtbvh_gpu_version() != nullptr);
}

void gpu_mode() {
  Vec3 grid[100];
  for (int x = 0; x <= 9; ++x)
    for (int y = 0; y <= 9; ++y) grid[x * 10 + y] = {float(x), float(y), 0.0f};
  RTAabb aabbs[27];
  float centers[27][4];
  for (int i = 0; i < 27; ++i) {
    aabbs[i] = box_of(&grid[3 * i]);
    for (int k = 0; k < 3; ++k) centers[i][k] = (aabbs[i].min[k] + aabbs[i].max[k]) * 0.5f;
    centers[i][3] = 0.0f;
  }
  RTBvh bvh{};
  RTMbvh mbvh{};
  CHECK(rtbvh::create_bvh(nullptr, 27, &centers[0][0], 16, 1, BvhType::BinnedSAH, &bvh) == ResultCode::Ok);
  rtbvh::free_bvh(bvh);
  CHECK(rtbvh::create_bvh(aabbs, 27, &centers[0][0], 16, 1, BvhType::BinnedSAH, &bvh) == ResultCode::Ok);
  CHECK(rtbvh::create_mbvh(bvh, &mbvh) == ResultCode::Ok);
  rtbvh::free_bvh(bvh);
  rtbvh::free_mbvh(mbvh);

  static const Vec3 quad[6] = {{-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};
  RTAabb qb[2] = {box_of(&quad[0]), box_of(&quad[3])};
  Vec3 qc[2];
  for (int i = 0; i < 2; ++i)
    qc[i] = {(qb[i].min[0] + qb[i].max[0]) * 0.5f, (qb[i].min[1] + qb[i].max[1]) * 0.5f,
             (qb[i].min[2] + qb[i].max[2]) * 0.5f};
  CHECK(rtbvh::create_bvh(qb, 2, &qc[0].x, sizeof(Vec3), 1, BvhType::BinnedSAH, &bvh) == ResultCode::Ok);
  CHECK(rtbvh::create_mbvh(bvh, &mbvh) == ResultCode::Ok);
  UserData ud{{0, 0, 0}, {0, 0, 1}, quad};
  float t = 1e26f;
  CHECK(rtbvh::intersect(bvh, &ud.origin.x, &ud.direction.x, &t, &ud, intersect_test) == ResultCode::Ok);
  CHECK(std::fabs(t - 1.0f) < 1.1920929e-7f);
  t = 1e26f;
  CHECK(rtbvh::intersect_mbvh(mbvh, &ud.origin.x, &ud.direction.x, &t, &ud, intersect_test) == ResultCode::Ok);
  CHECK(std::fabs(t - 1.0f) < 1.1920929e-7f);
  rtbvh::free_bvh(bvh);
  rtbvh::free_mbvh(mbvh);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) gpu_mode();
  else args_mode();
  if (failures) {
    std::fprintf(stderr, "%d checks failed\n", failures);
    return 1;
  }
  std::printf("abi_check.cpp ok\n");
  return 0;
}
