// Menu of in-block transform lengths with their compile-time radix schedules
// and block sizes.  Padded correlation lengths Nz are chosen so that Nz and Nz/2
// are both on this menu; every entry's block stages at most 20 complex values
// per thread per pass.
//
//   X(length, threads, radices...)
#pragma once

#define FPCC_SIZE_MENU(X)       \
  X(256, 128, 16, 16)           \
  X(320, 128, 16, 4, 5)         \
  X(384, 128, 16, 8, 3)         \
  X(512, 128, 16, 8, 4)         \
  X(640, 128, 16, 8, 5)         \
  X(768, 128, 16, 16, 3)        \
  X(1024, 128, 16, 16, 4)       \
  X(1280, 128, 16, 16, 5)       \
  X(1536, 128, 16, 8, 4, 3)     \
  X(2048, 128, 16, 16, 8)       \
  X(2560, 160, 16, 8, 4, 5)     \
  X(3072, 192, 16, 16, 4, 3)    \
  X(4096, 256, 16, 16, 16)      \
  X(5120, 320, 16, 16, 4, 5)    \
  X(6144, 384, 16, 16, 8, 3)    \
  X(8192, 512, 16, 16, 8, 4)    \
  X(10240, 640, 16, 16, 8, 5)   \
  X(12288, 768, 16, 16, 16, 3)  \
  X(16384, 1024, 16, 16, 16, 4) \
  X(20480, 1024, 8, 8, 8, 8, 5)

namespace fpcc {
// Lengths on the menu, ascending (host side).
constexpr int kMenu[] = {256,  320,  384,  512,  640,  768,   1024,  1280,  1536,  2048,
                         2560, 3072, 4096, 5120, 6144, 8192, 10240, 12288, 16384, 20480};
constexpr int kMenuLen = sizeof(kMenu) / sizeof(kMenu[0]);
inline bool on_menu(int n) {
  for (int i = 0; i < kMenuLen; i++)
    if (kMenu[i] == n) return true;
  return false;
}
}  // namespace fpcc
