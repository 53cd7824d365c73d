// Minimal stand-in for Boost.Serialization, enough for the reference's hot-path
// headers to compile (they only befriend `access` and name a few helpers).
// Written for the oracle build; no serialization is ever performed.
#pragma once
namespace boost { namespace serialization {
class access {};
template <class Archive, class T>
inline void split_member(Archive &, T &, const unsigned int) {}
template <class Archive, class T>
inline void split_free(Archive &, T &, const unsigned int) {}
template <class Base, class Derived>
inline Base &base_object(Derived &d) { return d; }
}}
