// sc_rec.cuh -- the FP32 geometry record of the mixed-precision form.
//
// A particle's record holds its centre relative to the centre of the cell it was
// sorted into, (x - (col+1/2) W, y - (row+1/2) H), and its shaft vector
// (A cos phi, A sin phi).  Positions stay in FP64; only this record is FP32.  The
// displacement of two particles whose cells are dc columns and dr rows apart is
// then rec_p - rec_q - (dc W, dr H): the periodic image is implied by the cell
// offset, so no box length enters the FP32 arithmetic.
#pragma once

#include <cuda_runtime.h>

namespace sc {

__device__ __forceinline__ float4 make_rec(double2 p, double phi, double A, int col, int row,
                                           double W, double H) {
  float sn, cs;
  sincosf((float)phi, &sn, &cs);
  float a = (float)A;
  return make_float4((float)(p.x - (col + 0.5) * W), (float)(p.y - (row + 0.5) * H), a * cs,
                     a * sn);
}

}  // namespace sc
