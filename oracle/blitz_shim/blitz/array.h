// blitz/array.h -- a minimal, eager stand-in for the parts of the Blitz++ 0.10
// Array API that zhubq/PhaseField's CPU time step uses.
//
// TEST INFRASTRUCTURE ONLY.  It exists so that the reference's own
// C++-openmp-cuda/src/{phase_field,solver,thermo_data,thermo_functor,write_data}.cpp
// compile unmodified into a checker library (oracle/build_oracle.py,
// build_ref_cpu) whose outputs pin the oracle's restatement of the phase
// sweep, the driver and the thermo evaluation.  Blitz++ itself is a
// third-party library that is neither vendored with the reference nor
// installed here; this header is written from its published interface
// (Blitz++ 0.10 manual: Array, Range, TinyVector, slicing, list
// initialisation, reductions), not from its source.
//
// What is provided, and the semantics kept:
//  * Array<T,N> with fortranArray storage: column-major (first index
//    fastest), every base 1.  Copy construction shares the data (a Blitz
//    reference); assignment from an array or a scalar copies values.
//  * Slicing with int / Range arguments: an int drops the rank, a Range keeps
//    it; the view keeps the original base, so A(Range(i,n)) is indexed from 1
//    (the reference's Sort_xyz adds i-1 to maxIndex of such a view).
//  * "A = a, b, c, ..." list initialisation in storage order; "A = x" alone
//    fills every element.
//  * Elementwise -A, A/x, A*B, exp(A), A<x, where(c, A, x); the reductions
//    sum, max and maxIndex (first maximum in storage order wins); cycleArrays.
// Expressions are evaluated eagerly, element by element, with the same
// per-element operations an expression template would apply, so results are
// bit-identical to a lazy evaluation under -ffp-contract=off.
#ifndef PF_BLITZ_SHIM_ARRAY_H
#define PF_BLITZ_SHIM_ARRAY_H

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <utility>
#include <vector>

namespace blitz {

// Storage tag: every array here uses the Fortran convention.
struct fortran_storage {};
static const fortran_storage fortranArray = {};

class Range {
public:
    Range(int first, int last) : first_(first), last_(last), all_(false) {}
    static Range all() {
        Range r(0, -1);
        r.all_ = true;
        return r;
    }
    int first_, last_;
    bool all_;
};

template <typename T, int N>
class TinyVector {
public:
    TinyVector() {
        for (int d = 0; d < N; d++) v_[d] = T();
    }
    explicit TinyVector(T x) {
        for (int d = 0; d < N; d++) v_[d] = x;
    }
    T &operator()(int d) { return v_[d]; }
    const T &operator()(int d) const { return v_[d]; }
    T &operator[](int d) { return v_[d]; }
    const T &operator[](int d) const { return v_[d]; }

private:
    T v_[N];
};

template <typename T, int N>
TinyVector<T, N> operator+(const TinyVector<T, N> &a, T b) {
    TinyVector<T, N> r;
    for (int d = 0; d < N; d++) r[d] = a[d] + b;
    return r;
}

template <typename T, int N>
class Array;

// "A = x" / "A = a, b, c, ...": one value fills the array; a comma list
// writes consecutive elements in storage order.
template <typename T, int N>
class ListInitializationSwitch {
public:
    ListInitializationSwitch(Array<T, N> &a, T x) : a_(a), first_(x), count_(1) {}
    ~ListInitializationSwitch() {
        if (count_ == 1) a_.fill(first_);
    }
    ListInitializationSwitch &operator,(T x) {
        if (count_ == 1) a_.linear(0) = first_;
        a_.linear(count_++) = x;
        return *this;
    }

private:
    Array<T, N> &a_;
    T first_;
    long count_;
};

template <typename T, int N>
class Array {
public:
    Array() { clear_shape(); }
    explicit Array(fortran_storage) { clear_shape(); }
    Array(int e0, fortran_storage) { allocate({e0}); }
    Array(int e0, int e1, fortran_storage) { allocate({e0, e1}); }
    Array(int e0, int e1, int e2, fortran_storage) { allocate({e0, e1, e2}); }
    Array(int e0, int e1, int e2, int e3, fortran_storage) { allocate({e0, e1, e2, e3}); }
    // Blitz semantics: a copy is a reference to the same data.
    Array(const Array &o) = default;

    void resize(int e0) { allocate({e0}); }
    void resize(int e0, int e1) { allocate({e0, e1}); }
    void resize(int e0, int e1, int e2) { allocate({e0, e1, e2}); }
    void resize(int e0, int e1, int e2, int e3) { allocate({e0, e1, e2, e3}); }

    // Element access (1-based).
    T &operator()(int i0) { return at({i0}); }
    T &operator()(int i0, int i1) { return at({i0, i1}); }
    T &operator()(int i0, int i1, int i2) { return at({i0, i1, i2}); }
    T &operator()(int i0, int i1, int i2, int i3) { return at({i0, i1, i2, i3}); }
    const T &operator()(int i0) const { return at({i0}); }
    const T &operator()(int i0, int i1) const { return at({i0, i1}); }
    const T &operator()(int i0, int i1, int i2) const { return at({i0, i1, i2}); }
    const T &operator()(int i0, int i1, int i2, int i3) const { return at({i0, i1, i2, i3}); }
    T &operator()(const TinyVector<int, 1> &i) { return at({i(0)}); }

    // Slices used by the reference: A(Range) on a 1-D array, A(i, all, all, all)
    // and A(all, i, j, k) on a 4-D array.
    Array<T, 1> operator()(Range r) const {
        static_assert(N == 1, "rank");
        Array<T, 1> v;
        v.share(*this);
        v.take_range(0, *this, 0, r);
        return v;
    }
    Array<T, 3> operator()(int i0, Range r1, Range r2, Range r3) const {
        static_assert(N == 4, "rank");
        Array<T, 3> v;
        v.share(*this);
        v.origin_ = origin_ + (long)(i0 - lb_[0]) * st_[0];
        v.take_range(0, *this, 1, r1);
        v.take_range(1, *this, 2, r2);
        v.take_range(2, *this, 3, r3);
        return v;
    }
    Array<T, 1> operator()(Range r0, int i1, int i2, int i3) const {
        static_assert(N == 4, "rank");
        Array<T, 1> v;
        v.share(*this);
        v.origin_ = origin_ + (long)(i1 - lb_[1]) * st_[1] + (long)(i2 - lb_[2]) * st_[2] +
                    (long)(i3 - lb_[3]) * st_[3];
        v.take_range(0, *this, 0, r0);
        return v;
    }

    ListInitializationSwitch<T, N> operator=(T x) { return ListInitializationSwitch<T, N>(*this, x); }
    Array &operator=(const Array &o) {
        assert(size() == o.size());
        for (long q = 0; q < size(); q++) linear(q) = o.linear(q);
        return *this;
    }

    T *data() { return origin_; }
    const T *data() const { return origin_; }
    int extent(int d) const { return ext_[d]; }
    int lbound(int d) const { return lb_[d]; }
    int ubound(int d) const { return lb_[d] + ext_[d] - 1; }
    long size() const {
        long s = 1;
        for (int d = 0; d < N; d++) s *= ext_[d];
        return s;
    }

    // q-th element in storage order (first index fastest).
    T &linear(long q) {
        long off = 0;
        for (int d = 0; d < N; d++) {
            off += (q % ext_[d]) * st_[d];
            q /= ext_[d];
        }
        return origin_[off];
    }
    const T &linear(long q) const { return const_cast<Array *>(this)->linear(q); }
    void fill(T x) {
        for (long q = 0; q < size(); q++) linear(q) = x;
    }
    void swap(Array &o) {
        std::swap(store_, o.store_);
        std::swap(origin_, o.origin_);
        for (int d = 0; d < N; d++) {
            std::swap(lb_[d], o.lb_[d]);
            std::swap(ext_[d], o.ext_[d]);
            std::swap(st_[d], o.st_[d]);
        }
    }
    // A fresh array of the same shape (base 1, contiguous).
    template <typename U>
    Array<U, N> same_shape() const {
        Array<U, N> r;
        std::vector<int> e(ext_, ext_ + N);
        r.allocate(e);
        return r;
    }

    // Internal state (public for the views and the elementwise helpers).
    std::shared_ptr<T> store_;  // the whole block (array deleter)
    T *origin_;
    int lb_[N], ext_[N];
    long st_[N];

    void clear_shape() {
        origin_ = nullptr;
        for (int d = 0; d < N; d++) {
            lb_[d] = 1;
            ext_[d] = 0;
            st_[d] = 0;
        }
    }
    void allocate(const std::vector<int> &e) {
        assert((int)e.size() == N);
        long s = 1;
        for (int d = 0; d < N; d++) {
            lb_[d] = 1;
            ext_[d] = e[d];
            st_[d] = s;
            s *= e[d];
        }
        store_ = std::shared_ptr<T>(new T[(size_t)(s > 0 ? s : 1)](), std::default_delete<T[]>());
        origin_ = store_.get();
    }
    template <int M>
    void share(const Array<T, M> &o) {
        store_ = o.store_;
        origin_ = o.origin_;
    }
    // Dimension d of this view takes dimension od of o restricted to r; the
    // view keeps o's base.
    template <int M>
    void take_range(int d, const Array<T, M> &o, int od, const Range &r) {
        const int first = r.all_ ? o.lb_[od] : r.first_;
        const int last = r.all_ ? o.lb_[od] + o.ext_[od] - 1 : r.last_;
        origin_ += (long)(first - o.lb_[od]) * o.st_[od];
        lb_[d] = o.lb_[od];
        ext_[d] = last - first + 1;
        st_[d] = o.st_[od];
    }

private:
    T &at(std::initializer_list<int> idx) {
        long off = 0;
        int d = 0;
        for (int i : idx) {
            assert(i >= lb_[d] && i < lb_[d] + ext_[d]);
            off += (long)(i - lb_[d]) * st_[d];
            d++;
        }
        return origin_[off];
    }
    const T &at(std::initializer_list<int> idx) const { return const_cast<Array *>(this)->at(idx); }
};

template <typename T, int N>
void cycleArrays(Array<T, N> &a, Array<T, N> &b) {
    a.swap(b);
}

// ---- elementwise operations (eager) ----
template <typename T, int N, typename F>
Array<T, N> map1(const Array<T, N> &a, F f) {
    Array<T, N> r = a.template same_shape<T>();
    for (long q = 0; q < a.size(); q++) r.linear(q) = f(a.linear(q));
    return r;
}
template <typename T, int N>
Array<T, N> operator-(const Array<T, N> &a) {
    return map1(a, [](T x) { return -x; });
}
template <typename T, int N>
Array<T, N> operator/(const Array<T, N> &a, double s) {
    return map1(a, [s](T x) { return x / s; });
}
template <typename T, int N>
Array<T, N> operator*(const Array<T, N> &a, const Array<T, N> &b) {
    assert(a.size() == b.size());
    Array<T, N> r = a.template same_shape<T>();
    for (long q = 0; q < a.size(); q++) r.linear(q) = a.linear(q) * b.linear(q);
    return r;
}
template <typename T, int N>
Array<T, N> exp(const Array<T, N> &a) {
    return map1(a, [](T x) { return std::exp(x); });
}
template <typename T, int N>
Array<bool, N> operator<(const Array<T, N> &a, T s) {
    Array<bool, N> r = a.template same_shape<bool>();
    for (long q = 0; q < a.size(); q++) r.linear(q) = a.linear(q) < s;
    return r;
}
template <typename T, int N>
Array<T, N> where(const Array<bool, N> &c, const Array<T, N> &a, T x) {
    Array<T, N> r = a.template same_shape<T>();
    for (long q = 0; q < a.size(); q++) r.linear(q) = c.linear(q) ? a.linear(q) : x;
    return r;
}

// ---- reductions, in storage order ----
template <typename T, int N>
T sum(const Array<T, N> &a) {
    T s = T();
    for (long q = 0; q < a.size(); q++) s += a.linear(q);
    return s;
}
template <typename T, int N>
T max(const Array<T, N> &a) {
    T m = -std::numeric_limits<T>::max();
    for (long q = 0; q < a.size(); q++)
        if (a.linear(q) > m) m = a.linear(q);
    return m;
}
// Index (in the array's own base) of the first maximum.
template <typename T>
TinyVector<int, 1> maxIndex(const Array<T, 1> &a) {
    T m = -std::numeric_limits<T>::max();
    int at = a.lbound(0);
    for (long q = 0; q < a.size(); q++)
        if (a.linear(q) > m) {
            m = a.linear(q);
            at = a.lbound(0) + (int)q;
        }
    return TinyVector<int, 1>(at);
}

}  // namespace blitz

#endif
