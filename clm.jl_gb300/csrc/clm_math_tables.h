// clm_math_tables.h — generated by gen_math_tables.py; do not edit.
#pragma once

CM_TABLE(CM_LOG_INVC, 128) = {
  0x1.54725e6bb82fep+0,
  0x1.52aff56a8054bp+0,
  0x1.50f22e111c4c5p+0,
  0x1.4f38f62dd4c9bp+0,
  0x1.4d843bedc2c4cp+0,
  0x1.4bd3edda68fe1p+0,
  0x1.4a27fad76014ap+0,
  0x1.4880522014880p+0,
  0x1.46dce34596066p+0,
  0x1.453d9e2c776cap+0,
  0x1.43a2730abee4dp+0,
  0x1.420b5265e5951p+0,
  0x1.40782d10e6566p+0,
  0x1.3ee8f42a5af07p+0,
  0x1.3d5d991aa75c6p+0,
  0x1.3bd60d9232955p+0,
  0x1.3a524387ac822p+0,
  0x1.38d22d366088ep+0,
  0x1.3755bd1c945eep+0,
  0x1.35dce5f9f2af8p+0,
  0x1.34679ace01346p+0,
  0x1.32f5ced6a1dfap+0,
  0x1.3187758e9ebb6p+0,
  0x1.301c82ac40260p+0,
  0x1.2eb4ea1fed14bp+0,
  0x1.2d50a012d50a0p+0,
  0x1.2bef98e5a3711p+0,
  0x1.2a91c92f3c105p+0,
  0x1.293725bb804a5p+0,
  0x1.27dfa38a1ce4dp+0,
  0x1.268b37cd60127p+0,
  0x1.2539d7e9177b2p+0,
  0x1.23eb79717605bp+0,
  0x1.22a0122a0122ap+0,
  0x1.21579804855e6p+0,
  0x1.2012012012012p+0,
  0x1.1ecf43c7fb84cp+0,
  0x1.1d8f5672e4abdp+0,
  0x1.1c522fc1ce059p+0,
  0x1.1b17c67f2bae3p+0,
  0x1.19e0119e0119ep+0,
  0x1.18ab083902bdbp+0,
  0x1.1778a191bd684p+0,
  0x1.1648d50fc3201p+0,
  0x1.151b9a3fdd5c9p+0,
  0x1.13f0e8d344724p+0,
  0x1.12c8b89edc0acp+0,
  0x1.11a3019a74826p+0,
  0x1.107fbbe011080p+0,
  0x1.0f5edfab325a2p+0,
  0x1.0e40655826011p+0,
  0x1.0d24456359e3ap+0,
  0x1.0c0a7868b4171p+0,
  0x1.0af2f722eecb5p+0,
  0x1.09ddba6af8360p+0,
  0x1.08cabb37565e2p+0,
  0x1.07b9f29b8eae2p+0,
  0x1.06ab59c7912fbp+0,
  0x1.059eea0727586p+0,
  0x1.04949cc1664c5p+0,
  0x1.038c6b78247fcp+0,
  0x1.02864fc7729e9p+0,
  0x1.0182436517a37p+0,
  0x1.0080402010080p+0,
  0x1.fe01fe01fe020p-1,
  0x1.fa11caa01fa12p-1,
  0x1.f6310aca0dbb5p-1,
  0x1.f25f644230ab5p-1,
  0x1.ee9c7f8458e02p-1,
  0x1.eae807aba01ebp-1,
  0x1.e741aa59750e4p-1,
  0x1.e3a9179dc1a73p-1,
  0x1.e01e01e01e01ep-1,
  0x1.dca01dca01dcap-1,
  0x1.d92f2231e7f8ap-1,
  0x1.d5cac807572b2p-1,
  0x1.d272ca3fc5b1ap-1,
  0x1.cf26e5c44bfc6p-1,
  0x1.cbe6d9601cbe7p-1,
  0x1.c8b265afb8a42p-1,
  0x1.c5894d10d4986p-1,
  0x1.c26b5392ea01cp-1,
  0x1.bf583ee868d8bp-1,
  0x1.bc4fd65883e7bp-1,
  0x1.b951e2b18ff23p-1,
  0x1.b65e2e3beee05p-1,
  0x1.b37484ad806cep-1,
  0x1.b094b31d922a4p-1,
  0x1.adbe87f94905ep-1,
  0x1.aaf1d2f87ebfdp-1,
  0x1.a82e65130e159p-1,
  0x1.a574107688a4ap-1,
  0x1.a2c2a87c51ca0p-1,
  0x1.a01a01a01a01ap-1,
  0x1.9d79f176b682dp-1,
  0x1.9ae24ea5510dap-1,
  0x1.9852f0d8ec0ffp-1,
  0x1.95cbb0be377aep-1,
  0x1.934c67f9b2ce6p-1,
  0x1.90d4f120190d5p-1,
  0x1.8e6527af1373fp-1,
  0x1.8bfce8062ff3ap-1,
  0x1.899c0f601899cp-1,
  0x1.87427bcc092b9p-1,
  0x1.84f00c2780614p-1,
  0x1.82a4a0182a4a0p-1,
  0x1.8060180601806p-1,
  0x1.7e225515a4f1dp-1,
  0x1.7beb3922e017cp-1,
  0x1.79baa6bb6398bp-1,
  0x1.77908119ac60dp-1,
  0x1.756cac201756dp-1,
  0x1.734f0c541fe8dp-1,
  0x1.713786d9c7c09p-1,
  0x1.6f26016f26017p-1,
  0x1.6d1a62681c861p-1,
  0x1.6b1490aa31a3dp-1,
  0x1.691473a88d0c0p-1,
  0x1.6719f3601671ap-1,
  0x1.6524f853b4aa3p-1,
  0x1.63356b88ac0dep-1,
  0x1.614b36831ae94p-1,
  0x1.5f66434292dfcp-1,
  0x1.5d867c3ece2a5p-1,
  0x1.5babcc647fa91p-1,
  0x1.59d61f123ccaap-1,
  0x1.5805601580560p-1,
  0x1.56397ba7c52e2p-1,
};
CM_TABLE(CM_LOG_LOGC, 128) = {
  -0x1.23ec5991eba49p-2,
  -0x1.1e9e1678899f5p-2,
  -0x1.1956d3b9bc2f9p-2,
  -0x1.14167ef367784p-2,
  -0x1.0edd060b78082p-2,
  -0x1.09aa572e6c6d4p-2,
  -0x1.047e60cde83b7p-2,
  -0x1.feb2233ea07cbp-3,
  -0x1.f474b134df228p-3,
  -0x1.ea4449f04aaf5p-3,
  -0x1.e020cc6235ab5p-3,
  -0x1.d60a17f903514p-3,
  -0x1.cc000c9db3c52p-3,
  -0x1.c2028ab17f9b5p-3,
  -0x1.b811730b823d4p-3,
  -0x1.ae2ca6f672bd8p-3,
  -0x1.a454082e6ab03p-3,
  -0x1.9a8778debaa3ap-3,
  -0x1.90c6db9fcbcdbp-3,
  -0x1.871213750e994p-3,
  -0x1.7d6903caf5acdp-3,
  -0x1.73cb9074fd14dp-3,
  -0x1.6a399dabbd383p-3,
  -0x1.60b3100b09474p-3,
  -0x1.5737cc9018cddp-3,
  -0x1.4dc7b897bc1c7p-3,
  -0x1.4462b9dc9b3dcp-3,
  -0x1.3b08b6757f2a7p-3,
  -0x1.31b994d3a4f86p-3,
  -0x1.28753bc11aba2p-3,
  -0x1.1f3b925f25d44p-3,
  -0x1.160c8024b27b0p-3,
  -0x1.0ce7ecdccc28bp-3,
  -0x1.03cdc0a51ec0dp-3,
  -0x1.f57bc7d9005dbp-4,
  -0x1.e3707ee30487bp-4,
  -0x1.d179788219362p-4,
  -0x1.bf968769fca18p-4,
  -0x1.adc77ee5aea8ep-4,
  -0x1.9c0c32d4d254dp-4,
  -0x1.8a6477a91dc29p-4,
  -0x1.78d02263d82d7p-4,
  -0x1.674f089365a78p-4,
  -0x1.55e10050e0382p-4,
  -0x1.4485e03dbdfb0p-4,
  -0x1.333d7f8183f4ap-4,
  -0x1.2207b5c7854a1p-4,
  -0x1.10e45b3cae829p-4,
  -0x1.ffa6911ab9309p-5,
  -0x1.dda8adc67ee59p-5,
  -0x1.bbcebfc68f424p-5,
  -0x1.9a187b573de81p-5,
  -0x1.788595a3577c8p-5,
  -0x1.5715c4c03cee1p-5,
  -0x1.35c8bfaa13069p-5,
  -0x1.149e3e4005a8dp-5,
  -0x1.e72bf2813ce6ap-6,
  -0x1.a55f548c5c427p-6,
  -0x1.63d6178690bbep-6,
  -0x1.228fb1fea2e0ap-6,
  -0x1.c317384c75f0dp-7,
  -0x1.41929f968330cp-7,
  -0x1.8121214586b02p-8,
  -0x1.0040155d5881ep-9,
  0x1.ff00aa2b10ba0p-9,
  0x1.7dc475f810a69p-7,
  0x1.3cea44346a584p-6,
  0x1.b9fc027af919ap-6,
  0x1.1b0d98923d97fp-5,
  0x1.58a5bafc8e4d3p-5,
  0x1.95c830ec8e3f2p-5,
  0x1.d276b8adb0b56p-5,
  0x1.075983598e471p-4,
  0x1.253f62f0a1417p-4,
  0x1.42edcbea646eep-4,
  0x1.60658a93750c4p-4,
  0x1.7da766d7b12d0p-4,
  0x1.9ab42462033aep-4,
  0x1.b78c82bb0eda0p-4,
  0x1.d4313d66cb35dp-4,
  0x1.f0a30c01162a4p-4,
  0x1.0671512ca596fp-3,
  0x1.14785846742acp-3,
  0x1.2266f190a5acdp-3,
  0x1.303d718e47fd5p-3,
  0x1.3dfc2b0ecc62ap-3,
  0x1.4ba36f39a55e5p-3,
  0x1.59338d9982085p-3,
  0x1.66acd4272ad51p-3,
  0x1.740f8f54037a3p-3,
  0x1.815c0a14357e9p-3,
  0x1.8e928de886d41p-3,
  0x1.9bb362e7dfb85p-3,
  0x1.a8becfc882f19p-3,
  0x1.b5b519e8fb5a6p-3,
  0x1.c2968558c18c2p-3,
  0x1.cf6354e09c5ddp-3,
  0x1.dc1bca0abec7bp-3,
  0x1.e8c0252aa5a60p-3,
  0x1.f550a564b7b37p-3,
  0x1.00e6c45ad501dp-2,
  0x1.071b85fcd590dp-2,
  0x1.0d46b579ab74bp-2,
  0x1.136870293a8b0p-2,
  0x1.1980d2dd4236fp-2,
  0x1.1f8ff9e48a2f3p-2,
  0x1.2596010df763ap-2,
  0x1.2b9303ab89d25p-2,
  0x1.31871c9544185p-2,
  0x1.3772662bfd85cp-2,
  0x1.3d54fa5c1f710p-2,
  0x1.432ef2a04e813p-2,
  0x1.49006804009d0p-2,
  0x1.4ec9732600269p-2,
  0x1.548a2c3add263p-2,
  0x1.5a42ab0f4cfe2p-2,
  0x1.5ff3070a793d4p-2,
  0x1.659b57303e1f2p-2,
  0x1.6b3bb2235943dp-2,
  0x1.70d42e2789236p-2,
  0x1.7664e1239dbcfp-2,
  0x1.7bede0a37afbfp-2,
  0x1.816f41da0d495p-2,
  0x1.86e919a330ba1p-2,
  0x1.8c5b7c858b48bp-2,
  0x1.91c67eb45a83ep-2,
  0x1.972a341135159p-2,
  0x1.9c86b02dc0862p-2,
};
CM_TABLE(CM_EXP_T, 64) = {
  0x1.0000000000000p+0,
  0x1.02c9a3e778061p+0,
  0x1.059b0d3158574p+0,
  0x1.0874518759bc8p+0,
  0x1.0b5586cf9890fp+0,
  0x1.0e3ec32d3d1a2p+0,
  0x1.11301d0125b51p+0,
  0x1.1429aaea92de0p+0,
  0x1.172b83c7d517bp+0,
  0x1.1a35beb6fcb75p+0,
  0x1.1d4873168b9aap+0,
  0x1.2063b88628cd6p+0,
  0x1.2387a6e756238p+0,
  0x1.26b4565e27cddp+0,
  0x1.29e9df51fdee1p+0,
  0x1.2d285a6e4030bp+0,
  0x1.306fe0a31b715p+0,
  0x1.33c08b26416ffp+0,
  0x1.371a7373aa9cbp+0,
  0x1.3a7db34e59ff7p+0,
  0x1.3dea64c123422p+0,
  0x1.4160a21f72e2ap+0,
  0x1.44e086061892dp+0,
  0x1.486a2b5c13cd0p+0,
  0x1.4bfdad5362a27p+0,
  0x1.4f9b2769d2ca7p+0,
  0x1.5342b569d4f82p+0,
  0x1.56f4736b527dap+0,
  0x1.5ab07dd485429p+0,
  0x1.5e76f15ad2148p+0,
  0x1.6247eb03a5585p+0,
  0x1.6623882552225p+0,
  0x1.6a09e667f3bcdp+0,
  0x1.6dfb23c651a2fp+0,
  0x1.71f75e8ec5f74p+0,
  0x1.75feb564267c9p+0,
  0x1.7a11473eb0187p+0,
  0x1.7e2f336cf4e62p+0,
  0x1.82589994cce13p+0,
  0x1.868d99b4492edp+0,
  0x1.8ace5422aa0dbp+0,
  0x1.8f1ae99157736p+0,
  0x1.93737b0cdc5e5p+0,
  0x1.97d829fde4e50p+0,
  0x1.9c49182a3f090p+0,
  0x1.a0c667b5de565p+0,
  0x1.a5503b23e255dp+0,
  0x1.a9e6b5579fdbfp+0,
  0x1.ae89f995ad3adp+0,
  0x1.b33a2b84f15fbp+0,
  0x1.b7f76f2fb5e47p+0,
  0x1.bcc1e904bc1d2p+0,
  0x1.c199bdd85529cp+0,
  0x1.c67f12e57d14bp+0,
  0x1.cb720dcef9069p+0,
  0x1.d072d4a07897cp+0,
  0x1.d5818dcfba487p+0,
  0x1.da9e603db3285p+0,
  0x1.dfc97337b9b5fp+0,
  0x1.e502ee78b3ff6p+0,
  0x1.ea4afa2a490dap+0,
  0x1.efa1bee615a27p+0,
  0x1.f50765b6e4540p+0,
  0x1.fa7c1819e90d8p+0,
};

#define CM_LN2N_HI (0x1.62e42fefa0000p-7)
#define CM_LN2N_LO (0x1.cf79abc9e3b3ap-46)
#define CM_INVLN2N (0x1.71547652b82fep+6)
#define CM_LN2_HI (0x1.62e42fefa3800p-1)
#define CM_LN2_LO (0x1.ef35793c76730p-45)
#define CM_INVLN10 (0x1.bcb7b1526e50ep-2)
#define CM_LOG_C2 (-0x1.0000000000000p-1)
#define CM_LOG_C3 (0x1.5555555555555p-2)
#define CM_LOG_C4 (-0x1.0000000000000p-2)
#define CM_LOG_C5 (0x1.999999999999ap-3)
#define CM_LOG_C6 (-0x1.5555555555555p-3)
#define CM_LOG_C7 (0x1.2492492492492p-3)
#define CM_EXP_C2 (0x1.0000000000000p-1)
#define CM_EXP_C3 (0x1.5555555555555p-3)
#define CM_EXP_C4 (0x1.5555555555555p-5)
#define CM_EXP_C5 (0x1.1111111111111p-7)
#define CM_EXP_C6 (0x1.6c16c16c16c17p-10)
#define CM_PIO2_HI (0x1.921fb54400000p+0)
#define CM_PIO2_MID (0x1.0b4611a600000p-34)
#define CM_PIO2_LO (0x1.3198a2e037073p-69)
#define CM_INVPIO2 (0x1.45f306dc9c883p-1)
#define CM_PIO4 (0x1.921fb54442d18p-1)
#define CM_DEG2RAD (0x1.1df46a2529d39p-6)
#define CM_SIN_S1 (-0x1.5555555555555p-3)
#define CM_SIN_S2 (0x1.1111111111111p-7)
#define CM_SIN_S3 (-0x1.a01a01a01a01ap-13)
#define CM_SIN_S4 (0x1.71de3a556c734p-19)
#define CM_SIN_S5 (-0x1.ae64567f544e4p-26)
#define CM_SIN_S6 (0x1.6124613a86d09p-33)
#define CM_SIN_S7 (-0x1.ae7f3e733b81fp-41)
#define CM_SIN_S8 (0x1.952c77030ad4ap-49)
#define CM_COS_C2 (0x1.5555555555555p-5)
#define CM_COS_C3 (-0x1.6c16c16c16c17p-10)
#define CM_COS_C4 (0x1.a01a01a01a01ap-16)
#define CM_COS_C5 (-0x1.27e4fb7789f5cp-22)
#define CM_COS_C6 (0x1.1eed8eff8d898p-29)
#define CM_COS_C7 (-0x1.93974a8c07c9dp-37)
#define CM_COS_C8 (0x1.ae7f3e733b81fp-45)
#define CM_ASIN_A1 (0x1.5555555555555p-3)
#define CM_ASIN_A2 (0x1.3333333333333p-4)
#define CM_ASIN_A3 (0x1.6db6db6db6db7p-5)
#define CM_ASIN_A4 (0x1.f1c71c71c71c7p-6)
#define CM_ASIN_A5 (0x1.6e8ba2e8ba2e9p-6)
#define CM_ASIN_A6 (0x1.1c4ec4ec4ec4fp-6)
#define CM_ASIN_A7 (0x1.c99999999999ap-7)
#define CM_ASIN_A8 (0x1.7a87878787878p-7)
#define CM_ASIN_A9 (0x1.3fde50d79435ep-7)
#define CM_ASIN_A10 (0x1.12ef3cf3cf3cfp-7)
#define CM_ASIN_A11 (0x1.df3bd37a6f4dfp-8)
#define CM_ASIN_A12 (0x1.a6863d70a3d71p-8)
#define CM_ASIN_A13 (0x1.782dda12f684cp-8)
#define CM_ASIN_A14 (0x1.51ba308d3dcb1p-8)
#define CM_ASIN_A15 (0x1.31683bdef7bdfp-8)
#define CM_ASIN_A16 (0x1.15ee9d45d1746p-8)
#define CM_ASIN_A17 (0x1.fcaf8fb6db6dbp-9)
#define CM_ASIN_A18 (0x1.d3d2a8e0dd67dp-9)
#define CM_ASIN_A19 (0x1.b026f57b13b14p-9)
#define CM_ASIN_A20 (0x1.90cb77f60c7cep-9)
#define CM_ASIN_A21 (0x1.750de64d7d05fp-9)
#define CM_ASIN_A22 (0x1.5c5f56efaaaabp-9)
#define CM_ASIN_A23 (0x1.464c0950f7d47p-9)
#define CM_ASIN_A24 (0x1.3275586c5f2f0p-9)
#define CM_ASIN_A25 (0x1.208d3570ae5a6p-9)
#define CM_ASIN_A26 (0x1.1052bc5fa960ap-9)
#define CM_ASIN_A27 (0x1.018f963c229bfp-9)
#define CM_PI_HI (0x1.921fb54442d18p+1)
#define CM_PI_LO (0x1.1a62633145c07p-53)
#define CM_PIO2_H (0x1.921fb54442d18p+0)
#define CM_PIO2_L (0x1.1a62633145c07p-54)
