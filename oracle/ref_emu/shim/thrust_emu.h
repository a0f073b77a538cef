// thrust_emu.h -- the few Thrust algorithms the reference calls, on host
// memory (TEST INFRASTRUCTURE for the reference emulation build).
#pragma once
#include <type_traits>

#include "colo_emu.h"

namespace thrust {
struct host_t {};
struct device_t {};
static host_t host;
static device_t device;

template <class T>
struct device_ptr {
    T* p;
    device_ptr() : p(nullptr) {}
    explicit device_ptr(T* q) : p(q) {}
    T* get() const { return p; }
    device_ptr operator+(long long n) const { return device_ptr(p + n); }
    device_ptr operator-(long long n) const { return device_ptr(p - n); }
    long long operator-(const device_ptr& o) const { return p - o.p; }
    T& operator*() const { return *p; }
};
template <class T>
device_ptr<T> device_pointer_cast(T* p) { return device_ptr<T>(p); }

template <class T> T* raw(T* p) { return p; }
template <class T> T* raw(device_ptr<T> p) { return p.p; }

// reduce with init = value_type() and plus on the value type
template <class It>
auto reduce(It first, It last) -> typename std::remove_reference<decltype(*raw(first))>::type {
    typedef typename std::remove_reference<decltype(*raw(first))>::type T;
    T s = T();
    auto* a = raw(first);
    auto* b = raw(last);
    for (auto* q = a; q < b; ++q) s = (T)(s + *q);
    if (colo_emu_hook_reduce) colo_emu_hook_reduce((size_t)(b > a ? b - a : 0), (unsigned long long)s);
    return s;
}
template <class It>
auto reduce(host_t, It first, It last) -> decltype(reduce(first, last)) {
    return reduce(first, last);
}

// stable sort of keys carrying values (thrust's radix sort is stable)
template <class K, class V>
void sort_by_key(K kfirst, K klast, V vfirst) {
    auto* k = raw(kfirst);
    auto* ke = raw(klast);
    auto* v = raw(vfirst);
    size_t n = (size_t)(ke - k);
    std::vector<size_t> idx(n);
    for (size_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return k[a] < k[b]; });
    typedef typename std::remove_reference<decltype(*k)>::type KT;
    typedef typename std::remove_reference<decltype(*v)>::type VT;
    std::vector<KT> kk(n);
    std::vector<VT> vv(n);
    for (size_t i = 0; i < n; ++i) {
        kk[i] = k[idx[i]];
        vv[i] = v[idx[i]];
    }
    for (size_t i = 0; i < n; ++i) {
        k[i] = kk[i];
        v[i] = vv[i];
    }
}

template <class K, class V>
void sort_by_key(host_t, K kfirst, K klast, V vfirst) {
    sort_by_key(kfirst, klast, vfirst);
}

// exclusive scan, init = input value_type(), accumulated in the input type
template <class It, class Ot>
Ot exclusive_scan(It first, It last, Ot result) {
    auto* a = raw(first);
    auto* b = raw(last);
    auto* o = raw(result);
    typedef typename std::remove_reference<decltype(*a)>::type T;
    T run = T();
    for (auto* q = a; q < b; ++q, ++o) {
        T v = *q;
        *o = run;
        run = (T)(run + v);
    }
    return result;
}
template <class It, class Ot>
Ot exclusive_scan(host_t, It first, It last, Ot result) {
    return exclusive_scan(first, last, result);
}
}  // namespace thrust
