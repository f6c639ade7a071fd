// FP64 -> FP32 conversion shared by the FP32 kernels.
#ifndef ANIGPU_FP_CONVERT_CUH
#define ANIGPU_FP_CONVERT_CUH

// FP64 -> FP32 with round-to-nearest-even in integer arithmetic.  GB300 runs FP64 (and
// the F64->F32 conversion) at a small fraction of its FP32 rate, so the FP32 paths keep
// FP64 instructions off their common path; zero, subnormal and out-of-range inputs go
// through the hardware conversion.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) return (b << 1) == 0 ? __uint_as_float(hi & 0x80000000u) : __double2float_rn(x);
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned f = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
    if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) f += 1u;
    return __uint_as_float(f);
}

#endif
