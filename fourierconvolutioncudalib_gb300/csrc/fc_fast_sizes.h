// Lengths covered by the register-resident kernels (all factors <= 16).
// Rows (x passes) go up to 4096, columns (y / z passes) up to 1024.  The
// batched persistent kernels, whose launch switches over every length they
// cover, keep to the power-of-two and microscope sizes (FC_BATCH_*); the
// single-volume kernels also cover common stack extents (FC_EXTRA_SIZES).
// Other lengths run on the generic kernels.
#pragma once
#define FC_FAST_COMMON_SIZES(X)                                                                                     \
  X(16) X(32) X(64) X(96) X(128) X(160) X(192) X(200) X(224) X(256) X(288) X(320) X(352) X(384) X(400) X(448) X(480) \
      X(512) X(576) X(640) X(768) X(960) X(1024)
#define FC_EXTRA_SIZES(X)                                                                                        \
  X(20) X(24) X(30) X(40) X(48) X(50) X(60) X(72) X(80) X(100) X(120) X(144) X(150) X(180) X(240) X(250) X(300) \
      X(360) X(500) X(600) X(720) X(800) X(900) X(1000)
#define FC_BATCH_ROW_SIZES(X) FC_FAST_COMMON_SIZES(X) X(2048) X(4096)
#define FC_BATCH_COL_SIZES(X) FC_FAST_COMMON_SIZES(X)
#define FC_ROW_SIZES(X) FC_BATCH_ROW_SIZES(X) FC_EXTRA_SIZES(X)
#define FC_COL_SIZES(X) FC_BATCH_COL_SIZES(X) FC_EXTRA_SIZES(X)
// column lengths served only by the wide in-place y pass (its exchange tile
// needs dynamic shared memory): 2048-row camera frames
#define FC_WIDE_ONLY_SIZES(X) X(2048)
