// Project-written stand-in: the reference names boost::heap::d_ary_heap only in
// one typedef of an out-of-scope index type and never instantiates it.
// Test infrastructure only.
#pragma once
namespace boost { namespace heap {
template <unsigned N> struct arity {};
template <class C> struct compare {};
template <class T, class A = void, class B = void> class d_ary_heap {};
}}  // namespace boost::heap
