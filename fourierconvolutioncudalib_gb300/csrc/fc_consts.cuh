// Generated by gen_consts.py -- DFT constants rounded once from double precision.
#pragma once

// cos(2*pi*j/P) and sin(2*pi*j/P), j = 0..P-1, for the odd prime butterflies.
template <int P> __device__ __forceinline__ float fc_dft_cos(int j);
template <int P> __device__ __forceinline__ float fc_dft_sin(int j);
template <> __device__ __forceinline__ float fc_dft_cos<3>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return -0.5f;
    case 2: return -0.5f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_sin<3>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.8660253882408142f;
    case 2: return -0.8660253882408142f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_cos<5>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.30901700258255005f;
    case 2: return -0.80901700258255f;
    case 3: return -0.80901700258255f;
    case 4: return 0.30901700258255005f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_sin<5>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.9510565400123596f;
    case 2: return 0.5877852439880371f;
    case 3: return -0.5877852439880371f;
    case 4: return -0.9510565400123596f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_cos<7>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.6234897971153259f;
    case 2: return -0.22252093255519867f;
    case 3: return -0.9009688496589661f;
    case 4: return -0.9009688496589661f;
    case 5: return -0.22252093255519867f;
    case 6: return 0.6234897971153259f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_sin<7>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.7818315029144287f;
    case 2: return 0.9749279022216797f;
    case 3: return 0.4338837265968323f;
    case 4: return -0.4338837265968323f;
    case 5: return -0.9749279022216797f;
    case 6: return -0.7818315029144287f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_cos<11>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.8412535190582275f;
    case 2: return 0.4154150187969208f;
    case 3: return -0.1423148363828659f;
    case 4: return -0.6548607349395752f;
    case 5: return -0.9594929814338684f;
    case 6: return -0.9594929814338684f;
    case 7: return -0.6548607349395752f;
    case 8: return -0.1423148363828659f;
    case 9: return 0.4154150187969208f;
    case 10: return 0.8412535190582275f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_sin<11>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.5406408309936523f;
    case 2: return 0.9096319675445557f;
    case 3: return 0.9898214340209961f;
    case 4: return 0.7557495832443237f;
    case 5: return 0.28173255920410156f;
    case 6: return -0.28173255920410156f;
    case 7: return -0.7557495832443237f;
    case 8: return -0.9898214340209961f;
    case 9: return -0.9096319675445557f;
    case 10: return -0.5406408309936523f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_cos<13>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.8854560256004333f;
    case 2: return 0.5680647492408752f;
    case 3: return 0.1205366775393486f;
    case 4: return -0.35460489988327026f;
    case 5: return -0.7485107779502869f;
    case 6: return -0.9709418416023254f;
    case 7: return -0.9709418416023254f;
    case 8: return -0.7485107779502869f;
    case 9: return -0.35460489988327026f;
    case 10: return 0.1205366775393486f;
    case 11: return 0.5680647492408752f;
    case 12: return 0.8854560256004333f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_dft_sin<13>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.4647231698036194f;
    case 2: return 0.8229838609695435f;
    case 3: return 0.9927088618278503f;
    case 4: return 0.9350162148475647f;
    case 5: return 0.6631226539611816f;
    case 6: return 0.23931565880775452f;
    case 7: return -0.23931565880775452f;
    case 8: return -0.6631226539611816f;
    case 9: return -0.9350162148475647f;
    case 10: return -0.9927088618278503f;
    case 11: return -0.8229838609695435f;
    case 12: return -0.4647231698036194f;
    default: return 0.0f;
  }
}

// cos(2*pi*j/R), sin(2*pi*j/R), j = 0..R-1, for the internal twiddles of the
// composite butterflies R = A*B (Cooley-Tukey inside the registers).
template <int R> __device__ __forceinline__ float fc_tw_cos(int j);
template <int R> __device__ __forceinline__ float fc_tw_sin(int j);
template <> __device__ __forceinline__ float fc_tw_cos<6>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.5f;
    case 2: return -0.5f;
    case 3: return -1.0f;
    case 4: return -0.5f;
    case 5: return 0.5f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<6>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.8660253882408142f;
    case 2: return 0.8660253882408142f;
    case 3: return 1.2246468525851679e-16f;
    case 4: return -0.8660253882408142f;
    case 5: return -0.8660253882408142f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_cos<9>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.7660444378852844f;
    case 2: return 0.1736481785774231f;
    case 3: return -0.5f;
    case 4: return -0.9396926164627075f;
    case 5: return -0.9396926164627075f;
    case 6: return -0.5f;
    case 7: return 0.1736481785774231f;
    case 8: return 0.7660444378852844f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<9>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.6427876353263855f;
    case 2: return 0.9848077297210693f;
    case 3: return 0.8660253882408142f;
    case 4: return 0.3420201539993286f;
    case 5: return -0.3420201539993286f;
    case 6: return -0.8660253882408142f;
    case 7: return -0.9848077297210693f;
    case 8: return -0.6427876353263855f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_cos<10>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.80901700258255f;
    case 2: return 0.30901700258255005f;
    case 3: return -0.30901700258255005f;
    case 4: return -0.80901700258255f;
    case 5: return -1.0f;
    case 6: return -0.80901700258255f;
    case 7: return -0.30901700258255005f;
    case 8: return 0.30901700258255005f;
    case 9: return 0.80901700258255f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<10>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.5877852439880371f;
    case 2: return 0.9510565400123596f;
    case 3: return 0.9510565400123596f;
    case 4: return 0.5877852439880371f;
    case 5: return 1.2246468525851679e-16f;
    case 6: return -0.5877852439880371f;
    case 7: return -0.9510565400123596f;
    case 8: return -0.9510565400123596f;
    case 9: return -0.5877852439880371f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_cos<12>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.8660253882408142f;
    case 2: return 0.5f;
    case 3: return 6.123234262925839e-17f;
    case 4: return -0.5f;
    case 5: return -0.8660253882408142f;
    case 6: return -1.0f;
    case 7: return -0.8660253882408142f;
    case 8: return -0.5f;
    case 9: return -1.8369701465288538e-16f;
    case 10: return 0.5f;
    case 11: return 0.8660253882408142f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<12>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.5f;
    case 2: return 0.8660253882408142f;
    case 3: return 1.0f;
    case 4: return 0.8660253882408142f;
    case 5: return 0.5f;
    case 6: return 1.2246468525851679e-16f;
    case 7: return -0.5f;
    case 8: return -0.8660253882408142f;
    case 9: return -1.0f;
    case 10: return -0.8660253882408142f;
    case 11: return -0.5f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_cos<14>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.9009688496589661f;
    case 2: return 0.6234897971153259f;
    case 3: return 0.22252093255519867f;
    case 4: return -0.22252093255519867f;
    case 5: return -0.6234897971153259f;
    case 6: return -0.9009688496589661f;
    case 7: return -1.0f;
    case 8: return -0.9009688496589661f;
    case 9: return -0.6234897971153259f;
    case 10: return -0.22252093255519867f;
    case 11: return 0.22252093255519867f;
    case 12: return 0.6234897971153259f;
    case 13: return 0.9009688496589661f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<14>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.4338837265968323f;
    case 2: return 0.7818315029144287f;
    case 3: return 0.9749279022216797f;
    case 4: return 0.9749279022216797f;
    case 5: return 0.7818315029144287f;
    case 6: return 0.4338837265968323f;
    case 7: return 1.2246468525851679e-16f;
    case 8: return -0.4338837265968323f;
    case 9: return -0.7818315029144287f;
    case 10: return -0.9749279022216797f;
    case 11: return -0.9749279022216797f;
    case 12: return -0.7818315029144287f;
    case 13: return -0.4338837265968323f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_cos<15>(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.9135454297065735f;
    case 2: return 0.6691306233406067f;
    case 3: return 0.30901700258255005f;
    case 4: return -0.10452846437692642f;
    case 5: return -0.5f;
    case 6: return -0.80901700258255f;
    case 7: return -0.9781476259231567f;
    case 8: return -0.9781476259231567f;
    case 9: return -0.80901700258255f;
    case 10: return -0.5f;
    case 11: return -0.10452846437692642f;
    case 12: return 0.30901700258255005f;
    case 13: return 0.6691306233406067f;
    case 14: return 0.9135454297065735f;
    default: return 0.0f;
  }
}
template <> __device__ __forceinline__ float fc_tw_sin<15>(int j) {
  switch (j) {
    case 0: return 0.0f;
    case 1: return 0.4067366421222687f;
    case 2: return 0.7431448101997375f;
    case 3: return 0.9510565400123596f;
    case 4: return 0.9945219159126282f;
    case 5: return 0.8660253882408142f;
    case 6: return 0.5877852439880371f;
    case 7: return 0.2079116851091385f;
    case 8: return -0.2079116851091385f;
    case 9: return -0.5877852439880371f;
    case 10: return -0.8660253882408142f;
    case 11: return -0.9945219159126282f;
    case 12: return -0.9510565400123596f;
    case 13: return -0.7431448101997375f;
    case 14: return -0.4067366421222687f;
    default: return 0.0f;
  }
}

// cos(2*pi*j/16), sin(2*pi*j/16) for the radix-16 internal twiddles.
#define FC_C16_1 0.9238795042037964f
#define FC_S16_1 0.3826834261417389f
#define FC_SQRT1_2 0.7071067690849304f

