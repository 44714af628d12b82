// Lengths covered by the register-resident kernels (all factors <= 16).
// Rows (x passes) go up to 4096, columns (y / z passes) up to 1024.
#pragma once
#define FC_FAST_COMMON_SIZES(X)                                                                                     \
  X(16) X(32) X(64) X(96) X(128) X(160) X(192) X(200) X(224) X(256) X(288) X(320) X(352) X(384) X(400) X(448) X(480) \
      X(512) X(576) X(640) X(768) X(960) X(1024)
#define FC_ROW_SIZES(X) FC_FAST_COMMON_SIZES(X) X(2048) X(4096)
#define FC_COL_SIZES(X) FC_FAST_COMMON_SIZES(X)
