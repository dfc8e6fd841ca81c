// Plane-wave app, boundary hook in the reference's plugin format (the
// signature of apps/hifu-beam/boundary.h:19-26), so that the reference's
// own fv.h/source.h run with it in the oracle's shim build.
// Oblique plane wave in a channel: zero-order extrapolation at both x ends,
// no-flux (mirror, normal momentum negated) walls at both y ends, corners
// zeroed.
#ifndef INC_BOUNDARY_H
#define INC_BOUNDARY_H

template <typename TTT>
__global__ void boundary(int *MDX, int *MDY, TTT *u1, TTT *u2, TTT *u3,
                         TTT *dx, TTT *dy, TTT *dt, TTT *T, GPUGD_VARSFD,
                         bool dstOut) {
  int i = threadIdx.x + blockIdx.x * blockDim.x;
  int j = threadIdx.y + blockIdx.y * blockDim.y;
  int offset = i + j * blockDim.x * gridDim.x;
  if (i > NX - 1 || j > NY - 1) return;
  int ir = i, jr = j;
  TTT sgn3 = Num1;
  if (i >= NX - 2) { ir = NX - 3; }
  else if (j >= NY - 2) { jr = 2 * (NY - 3) - j; sgn3 = -Num1; }
  else if (i <= 1) { ir = 2; }
  else if (j <= 1) { jr = 4 - j; sgn3 = -Num1; }
  if (dstOut) {
    u1[offset] = texAu1_read(&ir, &jr);
    u2[offset] = texAu2_read(&ir, &jr);
    u3[offset] = sgn3 * texAu3_read(&ir, &jr);
  } else {
    u1[offset] = texBu1_read(&ir, &jr);
    u2[offset] = texBu2_read(&ir, &jr);
    u3[offset] = sgn3 * texBu3_read(&ir, &jr);
  }
  if ((i <= 1 || i >= NX - 2) && (j <= 1 || j >= NY - 2)) {
    u1[offset] = Num0;
    u2[offset] = Num0;
    u3[offset] = Num0;
  }
}

#endif /* INC_BOUNDARY_H */
