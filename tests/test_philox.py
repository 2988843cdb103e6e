"""Philox4x32-10 of include/ncgb_philox.h against the Random123 known-answer
vectors (Salmon et al., SC'11; kat_vectors of the Random123 distribution)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "ncgb_philox.h"
#include <stdio.h>
static void run(uint32_t a,uint32_t b,uint32_t c,uint32_t d,uint32_t k0,uint32_t k1){
  uint32_t ctr[4]={a,b,c,d},o[4]; ncgb_philox4x32_10(ctr,k0,k1,o);
  printf("%08x %08x %08x %08x\n",o[0],o[1],o[2],o[3]); }
int main(void){
  run(0,0,0,0,0,0);
  run(0xffffffffu,0xffffffffu,0xffffffffu,0xffffffffu,0xffffffffu,0xffffffffu);
  run(0x243f6a88u,0x85a308d3u,0x13198a2eu,0x03707344u,0xa4093822u,0x299f31d0u);
  ncgb_rng r; ncgb_rng_init(&r,0,0,0,0);
  for (int i=0;i<3;++i) printf("%.17g\n", ncgb_rng_generate(&r));
  return 0; }
'''


def test_philox_known_answers(tmp_path):
    c = tmp_path / "k.c"
    c.write_text(SRC)
    exe = tmp_path / "k"
    subprocess.check_call(["gcc", "-std=c99", "-O2", "-I" + os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    assert out[0] == "6627e8d5 e169c58d bc57ac4c 9b00dbd8"
    assert out[1] == "408f276d 41c83b0e a20bc7c6 6d5451fd"
    assert out[2] == "d16cfe09 94fdcceb 5001e420 24126ea1"
    # draws: ((x0 | x1<<32) >> 11) + 1) * 2^-53 of block 0, then (x2, x3)
    x01 = 0x6627e8d5 | (0xe169c58d << 32)
    x23 = 0xbc57ac4c | (0x9b00dbd8 << 32)
    assert float(out[3]) == ((x01 >> 11) + 1) * 2.0 ** -53
    assert float(out[4]) == ((x23 >> 11) + 1) * 2.0 ** -53
    assert 0.0 < float(out[5]) <= 1.0
