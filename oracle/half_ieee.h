// IEEE-754 binary16 <-> binary32 conversion in portable C, written from the IEEE-754 definition.
// Test infrastructure: used only by the CPU oracle and by the reference-kernel harness (as the
// OpenCL C builtins vload_half / vstore_half_rte, which the OpenCL C specification defines as exact
// widening and round-to-nearest-even narrowing). The product's CUDA kernels use the hardware
// conversion instead; tests check the two agree.
#pragma once
#include <stdint.h>
#include <string.h>

static inline float half_bits_to_float(const uint16_t h) { // exact widening (every binary16 value is a binary32 value)
	const uint32_t sign = ((uint32_t)h&0x8000u)<<16;
	const uint32_t e = ((uint32_t)h>>10)&0x1Fu;
	uint32_t m = (uint32_t)h&0x3FFu;
	uint32_t x;
	if(e==0x1Fu) {
		x = sign|0x7F800000u|(m<<13); // inf / NaN (payload kept)
	} else if(e!=0u) {
		x = sign|((e+112u)<<23)|(m<<13); // normal: rebias 15 -> 127
	} else if(m==0u) {
		x = sign; // signed zero
	} else { // subnormal m*2^-24: normalise so bit 10 is set
		uint32_t shift = 0u;
		while(!(m&0x400u)) { m <<= 1; shift++; }
		x = sign|((113u-shift)<<23)|((m&0x3FFu)<<13);
	}
	float f;
	memcpy(&f, &x, 4);
	return f;
}

static inline uint16_t float_to_half_bits_rne(const float f) { // narrowing with round-to-nearest-even, overflow to inf
	uint32_t x;
	memcpy(&x, &f, 4);
	const uint32_t sign = (x>>16)&0x8000u;
	const uint32_t a = x&0x7FFFFFFFu;
	if(a>=0x7F800000u) return (uint16_t)(sign|0x7C00u|(a>0x7F800000u ? 0x200u|((a>>13)&0x3FFu) : 0u)); // inf / NaN
	if(a>=0x477FF000u) return (uint16_t)(sign|0x7C00u); // |f| >= 65520 rounds to inf
	if(a>=0x38800000u) { // result is a normal half: |f| >= 2^-14
		const uint32_t r = a-0x38000000u; // rebias exponent 127 -> 15 (stays in the same bit position)
		const uint32_t rounded = r+0x0FFFu+((r>>13)&1u); // round the 13 dropped mantissa bits to nearest even
		return (uint16_t)(sign|(rounded>>13));
	}
	// result is subnormal or zero: count of 2^-24 units, k = round_even(M * 2^(e-126))
	const uint32_t e = a>>23;
	if(e<102u) return (uint16_t)sign; // |f| < 2^-25 (and float subnormals) round to zero
	const uint32_t M = (a&0x7FFFFFu)|0x800000u;
	const uint32_t s = 126u-e; // 14..24
	uint32_t k = M>>s;
	const uint32_t rem = M&((1u<<s)-1u), halfway = 1u<<(s-1u);
	if(rem>halfway||(rem==halfway&&(k&1u))) k++;
	return (uint16_t)(sign|k);
}
