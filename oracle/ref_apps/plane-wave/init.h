// Plane-wave app, init hook in the reference's plugin format
// (apps/taylor-angle-xy/init.h:17-29): u1 = A sin(2 pi FREC (x cos a +
// y sin a)), (u2, u3) = u1 (cos a, sin a), evaluated in double.
#ifndef INC_INIT_H
#define INC_INIT_H

template <typename TTT>
void init(TTT *u1, TTT *u2, TTT *u3, TTT *dx, TTT *dy, TTT *dt, GPUGD_VARSFD) {
  const double ddx = PW_XMAX / double(NX - 1), ddy = PW_YMAX / double(NY - 1);
  for (int i = 0; i < NX; i++) {
    for (int j = 0; j < NY; j++) {
      double ph = 2.0 * 3.141592653589793 * PW_FREC *
                  (double(i) * ddx * cos(PW_ANGLE) + double(j) * ddy * sin(PW_ANGLE));
      double a = PW_AMPL * sin(ph);
      u1[i + j * NX] = TTT(a);
      u2[i + j * NX] = TTT(a * cos(PW_ANGLE));
      u3[i + j * NX] = TTT(a * sin(PW_ANGLE));
    }
  }
}

#endif /* INC_INIT_H */
