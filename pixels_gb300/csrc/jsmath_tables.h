// Generated by gen_jsmath_tables.py (mpmath, 200-bit); do not edit.
#pragma once

// Each table exists twice: a __device__ copy for GPU code and a host copy;
// PX_TAB(name) picks the one for the side being compiled.
#if defined(__CUDACC__)
#define PX_DEVTAB __device__ const
#else
#define PX_DEVTAB const
#endif
#if defined(__CUDA_ARCH__)
#define PX_TAB(name) name##_d
#else
#define PX_TAB(name) name##_h
#endif

// pi/2 as three doubles (Cody-Waite reduction pieces)
#define PX_PIO2_1 0x1.921fb54442d18p+0
#define PX_PIO2_2 0x1.1a62633145c07p-54
#define PX_PIO2_3 -0x1.f1976b7ed8fbcp-110
#define PX_PI_HI 0x1.921fb54442d18p+1
#define PX_PI_LO 0x1.1a62633145c07p-53
#define PX_PIO2_HI 0x1.921fb54442d18p+0
#define PX_PIO2_LO 0x1.1a62633145c07p-54
#define PX_2OPI 0x1.45f306dc9c883p-1

// 1/n! for n = 0..30 as double-double (hi, lo)
static PX_DEVTAB double PX_INVFACT_d[31][2] = {
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.0000000000000p-1, 0x0.0p+0},
  {0x1.5555555555555p-3, 0x1.5555555555555p-57},
  {0x1.5555555555555p-5, 0x1.5555555555555p-59},
  {0x1.1111111111111p-7, 0x1.1111111111111p-63},
  {0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65},
  {0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73},
  {0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76},
  {0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73},
  {0x1.27e4fb7789f5cp-22, 0x1.cbbc05b4fa99ap-76},
  {0x1.ae64567f544e4p-26, -0x1.c062e06d1f209p-80},
  {0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83},
  {0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87},
  {0x1.93974a8c07c9dp-37, 0x1.05d6f8a2efd1fp-92},
  {0x1.ae7f3e733b81fp-41, 0x1.1d8656b0ee8cbp-97},
  {0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101},
  {0x1.952c77030ad4ap-49, 0x1.ac981465ddc6cp-103},
  {0x1.6827863b97d97p-53, 0x1.eec01221a8b0bp-107},
  {0x1.2f49b46814157p-57, 0x1.2650f61dbdcb4p-112},
  {0x1.e542ba4020225p-62, 0x1.ea72b4afe3c2fp-120},
  {0x1.71b8ef6dcf572p-66, -0x1.d043ae40c4647p-120},
  {0x1.0ce396db7f853p-70, -0x1.aebcdbd20331cp-124},
  {0x1.761b41316381ap-75, -0x1.3423c7d91404fp-130},
  {0x1.f2cf01972f578p-80, -0x1.9ada5fcc1ab14p-135},
  {0x1.3f3ccdd165fa9p-84, -0x1.58ddadf344487p-139},
  {0x1.88e85fc6a4e5ap-89, -0x1.71c37ebd16540p-143},
  {0x1.d1ab1c2dccea3p-94, 0x1.054d0c78aea14p-149},
  {0x1.0a18a2635085dp-98, 0x1.b9e2e28e1aa54p-153},
  {0x1.259f98b4358adp-103, 0x1.eaf8c39dd9bc5p-157},
  {0x1.3932c5047d60ep-108, 0x1.832b7b530a627p-162},
};
static const double PX_INVFACT_h[31][2] = {
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.0000000000000p-1, 0x0.0p+0},
  {0x1.5555555555555p-3, 0x1.5555555555555p-57},
  {0x1.5555555555555p-5, 0x1.5555555555555p-59},
  {0x1.1111111111111p-7, 0x1.1111111111111p-63},
  {0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65},
  {0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73},
  {0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76},
  {0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73},
  {0x1.27e4fb7789f5cp-22, 0x1.cbbc05b4fa99ap-76},
  {0x1.ae64567f544e4p-26, -0x1.c062e06d1f209p-80},
  {0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83},
  {0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87},
  {0x1.93974a8c07c9dp-37, 0x1.05d6f8a2efd1fp-92},
  {0x1.ae7f3e733b81fp-41, 0x1.1d8656b0ee8cbp-97},
  {0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101},
  {0x1.952c77030ad4ap-49, 0x1.ac981465ddc6cp-103},
  {0x1.6827863b97d97p-53, 0x1.eec01221a8b0bp-107},
  {0x1.2f49b46814157p-57, 0x1.2650f61dbdcb4p-112},
  {0x1.e542ba4020225p-62, 0x1.ea72b4afe3c2fp-120},
  {0x1.71b8ef6dcf572p-66, -0x1.d043ae40c4647p-120},
  {0x1.0ce396db7f853p-70, -0x1.aebcdbd20331cp-124},
  {0x1.761b41316381ap-75, -0x1.3423c7d91404fp-130},
  {0x1.f2cf01972f578p-80, -0x1.9ada5fcc1ab14p-135},
  {0x1.3f3ccdd165fa9p-84, -0x1.58ddadf344487p-139},
  {0x1.88e85fc6a4e5ap-89, -0x1.71c37ebd16540p-143},
  {0x1.d1ab1c2dccea3p-94, 0x1.054d0c78aea14p-149},
  {0x1.0a18a2635085dp-98, 0x1.b9e2e28e1aa54p-153},
  {0x1.259f98b4358adp-103, 0x1.eaf8c39dd9bc5p-157},
  {0x1.3932c5047d60ep-108, 0x1.832b7b530a627p-162},
};

// atan(k/32) for k = 0..32 as double-double (hi, lo)
static PX_DEVTAB double PX_ATAN_TAB_d[33][2] = {
  {0x0.0p+0, 0x0.0p+0},
  {0x1.ffd55bba97625p-6, -0x1.5ec431444912cp-60},
  {0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60},
  {0x1.7ee182602f10fp-4, -0x1.cfb654c0c3d98p-58},
  {0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59},
  {0x1.3d6eee8c6626cp-3, 0x1.61a3b0ce9281bp-57},
  {0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58},
  {0x1.b90d7529260a2p-3, 0x1.17b10d2e0e5abp-61},
  {0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57},
  {0x1.18bf5a30bf178p-2, 0x1.30ca4748b1bf9p-57},
  {0x1.362773707ebccp-2, -0x1.963a544b672d8p-57},
  {0x1.530ad9951cd4ap-2, -0x1.2566480884082p-57},
  {0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56},
  {0x1.8b24d394a1b25p-2, 0x1.b6d0ba3748fa8p-56},
  {0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56},
  {0x1.c0db4c94ec9f0p-2, -0x1.cc1ce70934c34p-56},
  {0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56},
  {0x1.f40dd0b541418p-2, -0x1.a3992dc382a23p-57},
  {0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56},
  {0x1.1255d9bfbd2a9p-1, -0x1.2bdaee1c0ee35p-58},
  {0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58},
  {0x1.2958e59308e31p-1, -0x1.09e73b0c6c087p-56},
  {0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55},
  {0x1.3f13fb89e96f4p-1, 0x1.ecf8b492644f0p-56},
  {0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56},
  {0x1.538f57b89061fp-1, -0x1.1bb74abda520cp-55},
  {0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57},
  {0x1.66d663923e087p-1, -0x1.6ea6febe8bbbap-56},
  {0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56},
  {0x1.78f6bbd5d315ep-1, 0x1.406a089803740p-55},
  {0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56},
  {0x1.89ff5ff57f1f8p-1, -0x1.55b9a5e177a1bp-55},
  {0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55},
};
static const double PX_ATAN_TAB_h[33][2] = {
  {0x0.0p+0, 0x0.0p+0},
  {0x1.ffd55bba97625p-6, -0x1.5ec431444912cp-60},
  {0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60},
  {0x1.7ee182602f10fp-4, -0x1.cfb654c0c3d98p-58},
  {0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59},
  {0x1.3d6eee8c6626cp-3, 0x1.61a3b0ce9281bp-57},
  {0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58},
  {0x1.b90d7529260a2p-3, 0x1.17b10d2e0e5abp-61},
  {0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57},
  {0x1.18bf5a30bf178p-2, 0x1.30ca4748b1bf9p-57},
  {0x1.362773707ebccp-2, -0x1.963a544b672d8p-57},
  {0x1.530ad9951cd4ap-2, -0x1.2566480884082p-57},
  {0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56},
  {0x1.8b24d394a1b25p-2, 0x1.b6d0ba3748fa8p-56},
  {0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56},
  {0x1.c0db4c94ec9f0p-2, -0x1.cc1ce70934c34p-56},
  {0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56},
  {0x1.f40dd0b541418p-2, -0x1.a3992dc382a23p-57},
  {0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56},
  {0x1.1255d9bfbd2a9p-1, -0x1.2bdaee1c0ee35p-58},
  {0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58},
  {0x1.2958e59308e31p-1, -0x1.09e73b0c6c087p-56},
  {0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55},
  {0x1.3f13fb89e96f4p-1, 0x1.ecf8b492644f0p-56},
  {0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56},
  {0x1.538f57b89061fp-1, -0x1.1bb74abda520cp-55},
  {0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57},
  {0x1.66d663923e087p-1, -0x1.6ea6febe8bbbap-56},
  {0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56},
  {0x1.78f6bbd5d315ep-1, 0x1.406a089803740p-55},
  {0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56},
  {0x1.89ff5ff57f1f8p-1, -0x1.55b9a5e177a1bp-55},
  {0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55},
};

// 1/(2n+1) for n = 0..15 as double-double (hi, lo)
static PX_DEVTAB double PX_INVODD_d[16][2] = {
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.5555555555555p-2, 0x1.5555555555555p-56},
  {0x1.999999999999ap-3, -0x1.999999999999ap-57},
  {0x1.2492492492492p-3, 0x1.2492492492492p-57},
  {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58},
  {0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59},
  {0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58},
  {0x1.1111111111111p-4, 0x1.1111111111111p-60},
  {0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61},
  {0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59},
  {0x1.8618618618618p-5, 0x1.8618618618618p-59},
  {0x1.642c8590b2164p-5, 0x1.642c8590b2164p-60},
  {0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61},
  {0x1.2f684bda12f68p-5, 0x1.2f684bda12f68p-59},
  {0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61},
  {0x1.0842108421084p-5, 0x1.0842108421084p-60},
};
static const double PX_INVODD_h[16][2] = {
  {0x1.0000000000000p+0, 0x0.0p+0},
  {0x1.5555555555555p-2, 0x1.5555555555555p-56},
  {0x1.999999999999ap-3, -0x1.999999999999ap-57},
  {0x1.2492492492492p-3, 0x1.2492492492492p-57},
  {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58},
  {0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59},
  {0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58},
  {0x1.1111111111111p-4, 0x1.1111111111111p-60},
  {0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61},
  {0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59},
  {0x1.8618618618618p-5, 0x1.8618618618618p-59},
  {0x1.642c8590b2164p-5, 0x1.642c8590b2164p-60},
  {0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61},
  {0x1.2f684bda12f68p-5, 0x1.2f684bda12f68p-59},
  {0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61},
  {0x1.0842108421084p-5, 0x1.0842108421084p-60},
};
