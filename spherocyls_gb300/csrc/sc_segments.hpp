// sc_segments.hpp -- distance between two spines (segments), for the placement
// rules of the configuration generators (host and device).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SC_HD __host__ __device__ __forceinline__
#else
#define SC_HD inline
#endif

namespace sc_seg {

SC_HD double cross(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

// distance from point (px,py) to the segment c + t*u, t in [-1, 1]
SC_HD double point_seg(double px, double py, double cx, double cy, double ux, double uy) {
  double uu = ux * ux + uy * uy;
  double t = 0.0;
  if (uu > 0) {
    t = ((px - cx) * ux + (py - cy) * uy) / uu;
    t = t < -1 ? -1 : (t > 1 ? 1 : t);
  }
  double dx = px - (cx + t * ux), dy = py - (cy + t * uy);
  return sqrt(dx * dx + dy * dy);
}

// distance between segments a + s*u and b + t*v (s, t in [-1, 1]): zero when they
// cross, else the least endpoint-to-segment distance
SC_HD double seg_seg(double ax, double ay, double ux, double uy, double bx, double by, double vx,
                     double vy) {
  double p0x = ax - ux, p0y = ay - uy, p1x = ax + ux, p1y = ay + uy;
  double q0x = bx - vx, q0y = by - vy, q1x = bx + vx, q1y = by + vy;
  double d1 = cross(q1x - q0x, q1y - q0y, p0x - q0x, p0y - q0y);
  double d2 = cross(q1x - q0x, q1y - q0y, p1x - q0x, p1y - q0y);
  double d3 = cross(p1x - p0x, p1y - p0y, q0x - p0x, q0y - p0y);
  double d4 = cross(p1x - p0x, p1y - p0y, q1x - p0x, q1y - p0y);
  if (((d1 > 0 && d2 < 0) || (d1 < 0 && d2 > 0)) && ((d3 > 0 && d4 < 0) || (d3 < 0 && d4 > 0)))
    return 0.0;
  double m = point_seg(p0x, p0y, bx, by, vx, vy);
  m = fmin(m, point_seg(p1x, p1y, bx, by, vx, vy));
  m = fmin(m, point_seg(q0x, q0y, ax, ay, ux, uy));
  m = fmin(m, point_seg(q1x, q1y, ax, ay, ux, uy));
  return m;
}

}  // namespace sc_seg
