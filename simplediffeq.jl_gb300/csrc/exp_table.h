/* generated by gen_exptab.py: 2^(j/32) = lead + trail for j = 0..31, the exponential table of the
 * FP64 step-size controller, and ln2/32 in two parts */
#pragma once
#ifndef GBODE_EXPTAB_SPACE
#define GBODE_EXPTAB_SPACE static const
#endif
#define GBODE_EXP_INV_L 0x1.71547652b82fep+5 /* 32/ln 2 */
#define GBODE_EXP_L_LEAD 0x1.62e42fefa3800p-6 /* ln2/32, 42 significant bits */
#define GBODE_EXP_L_TRAIL 0x1.ef35793c76730p-50
GBODE_EXPTAB_SPACE double kExpTab[32][2] = {
    {0x1.0000000000000p+0, 0x0.0p+0},
    {0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55},
    {0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54},
    {0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54},
    {0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55},
    {0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54},
    {0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54},
    {0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55},
    {0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55},
    {0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54},
    {0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55},
    {0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59},
    {0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56},
    {0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55},
    {0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54},
    {0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54},
    {0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54},
    {0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55},
    {0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55},
    {0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54},
    {0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54},
    {0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57},
    {0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56},
    {0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54},
    {0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54},
    {0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56},
    {0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55},
    {0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56},
    {0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55},
    {0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54},
    {0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54},
    {0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54},
};
