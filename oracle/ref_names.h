// Symbol suffix per precision: _f64 for the DOUBLE build, _f32 for SINGLE.
#pragma once
#define HXREF_CAT2(a, b) a##b
#define HXREF_CAT(a, b) HXREF_CAT2(a, b)
#ifdef HXREF_SINGLE
#define HXREF_NAME(x) HXREF_CAT(x, _f32)
#else
#define HXREF_NAME(x) HXREF_CAT(x, _f64)
#endif
