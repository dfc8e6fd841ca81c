// Focused-beam app, boundary hook in the reference's plugin format (the
// signature of apps/hifu-beam/boundary.h:19-26). A continuous-wave source
// on the left edge over |j - FB_CENTER| < FB_HALFAP, focused at ISPF points
// with the hifu phase law phi = dx j'^2 / (2 ISPF) (hifu boundary.h:88),
// amplitude ramped linearly over the first periods; zero-order
// extrapolation on every other edge; corners zeroed.
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
  if (i >= NX - 2) { ir = NX - 3; }
  else if (j >= NY - 2) { jr = NY - 3; }
  else if (i <= 1) { ir = 2; }
  else if (j <= 1) { jr = 2; }
  if (dstOut) {
    u1[offset] = texAu1_read(&ir, &jr);
    u2[offset] = texAu2_read(&ir, &jr);
    u3[offset] = texAu3_read(&ir, &jr);
  } else {
    u1[offset] = texBu1_read(&ir, &jr);
    u2[offset] = texBu2_read(&ir, &jr);
    u3[offset] = texBu3_read(&ir, &jr);
  }
  if (i <= 1 && j > 1 && j < NY - 2) {
    TTT jp = TTT(j) - FB_CENTER;
    if (fabs(jp) < FB_HALFAP && (*MDX) == 0) {
      TTT jp2 = jp * jp;
      TTT nudenom = sqrt(jp2 + ISPF * ISPF);
      TTT nux = ISPF / nudenom;
      TTT nuy = -jp / nudenom;
      TTT phi = ((*dx) * jp2) / (Num2 * ISPF);
      TTT t = (*T) + phi;
      TTT ramp = getmin(getmax(t * FB_RAMP, Num0), Num1);
      TTT pack = AMPL * ramp * sin(ISPW * t);
      u1[offset] = pack;
      u2[offset] = nux * pack * (pack + Num1);
      u3[offset] = nuy * pack * (pack + Num1);
    }
  }
  if ((i <= 1 || i >= NX - 2) && (j <= 1 || j >= NY - 2)) {
    u1[offset] = Num0;
    u2[offset] = Num0;
    u3[offset] = Num0;
  }
}

#endif /* INC_BOUNDARY_H */
