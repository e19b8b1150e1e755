// device_atomic_functions.h — host stand-in for the CUDA atomics the reference's kernels call (TEST INFRASTRUCTURE
// ONLY). It shadows the toolkit header of the same name when the reference is compiled as host C++: each function
// performs the read-modify-write atomically on the host (GCC __atomic builtins) and returns the old value, as the
// CUDA functions do.
#pragma once

#include <cstdint>

inline unsigned int atomicAdd(unsigned int* a, unsigned int v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
inline int atomicAdd(int* a, int v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
inline unsigned long long atomicAdd(unsigned long long* a, unsigned long long v) {
    return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST);
}
inline float atomicAdd(float* a, float v) {
    float old, upd;
    __atomic_load(a, &old, __ATOMIC_SEQ_CST);
    do {
        upd = old + v;
    } while (!__atomic_compare_exchange(a, &old, &upd, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST));
    return old;
}
inline unsigned int atomicSub(unsigned int* a, unsigned int v) { return __atomic_fetch_sub(a, v, __ATOMIC_SEQ_CST); }
inline int atomicSub(int* a, int v) { return __atomic_fetch_sub(a, v, __ATOMIC_SEQ_CST); }
inline unsigned int atomicExch(unsigned int* a, unsigned int v) { return __atomic_exchange_n(a, v, __ATOMIC_SEQ_CST); }
inline unsigned int atomicCAS(unsigned int* a, unsigned int cmp, unsigned int v) {
    __atomic_compare_exchange_n(a, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp;
}
inline unsigned int atomicMin(unsigned int* a, unsigned int v) {
    unsigned int old = __atomic_load_n(a, __ATOMIC_SEQ_CST);
    while (v < old && !__atomic_compare_exchange_n(a, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
    }
    return old;
}
