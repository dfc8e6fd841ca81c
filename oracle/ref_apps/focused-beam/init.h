// Focused-beam app, init hook in the reference's plugin format: a medium at
// rest (as apps/hifu-beam/init.h:16-25).
#ifndef INC_INIT_H
#define INC_INIT_H

template <typename TTT>
void init(TTT *u1, TTT *u2, TTT *u3, TTT *dx, TTT *dy, TTT *dt, GPUGD_VARSFD) {
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++) {
      u1[i + j * NX] = Num0;
      u2[i + j * NX] = Num0;
      u3[i + j * NX] = Num0;
    }
}

#endif /* INC_INIT_H */
