/* Minimal stand-in for boost::iterator_facade, enough for the random-access
 * node_iter of helper_files_common/csr4matrix.hpp:84-130.  Used only to build
 * oracle/_ref (Boost is not installed here). */
#pragma once
#include <cstddef>
#include <iterator>
#include <type_traits>
namespace boost {
struct random_access_traversal_tag {};
struct iterator_core_access {
    template <class F> static typename F::reference deref(const F& f) { return f.dereference(); }
    template <class F> static void inc(F& f) { f.increment(); }
    template <class F> static void dec(F& f) { f.decrement(); }
    template <class F, class D> static void adv(F& f, D n) { f.advance(n); }
    template <class F> static bool eq(const F& a, const F& b) { return a.equal(b); }
    template <class F> static typename F::difference_type dist(const F& a, const F& b) { return a.distance_to(b); }
};
template <class Derived, class Value, class Category, class Reference = Value&, class Difference = std::ptrdiff_t>
class iterator_facade {
public:
    typedef typename std::remove_const<Value>::type value_type;
    typedef Reference reference;
    typedef Difference difference_type;
    typedef Value* pointer;
    typedef std::random_access_iterator_tag iterator_category;
    reference operator*() const { return iterator_core_access::deref(d()); }
    pointer operator->() const { return &iterator_core_access::deref(d()); }
    Derived& operator++() { iterator_core_access::inc(d()); return d(); }
    Derived operator++(int) { Derived t(d()); iterator_core_access::inc(d()); return t; }
    Derived& operator--() { iterator_core_access::dec(d()); return d(); }
    Derived& operator+=(difference_type n) { iterator_core_access::adv(d(), n); return d(); }
    Derived operator+(difference_type n) const { Derived t(d()); iterator_core_access::adv(t, n); return t; }
    difference_type operator-(const Derived& o) const { return iterator_core_access::dist(o, d()); }
    bool operator==(const Derived& o) const { return iterator_core_access::eq(d(), o); }
    bool operator!=(const Derived& o) const { return !iterator_core_access::eq(d(), o); }
private:
    Derived& d() { return *static_cast<Derived*>(this); }
    const Derived& d() const { return *static_cast<const Derived*>(this); }
};
}  // namespace boost
