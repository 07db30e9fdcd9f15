// ref_boost.hpp - stand-in for the Boost.Serialization names that nav24's camera models declare
// (TEST INFRASTRUCTURE: only the reference-pin recipe, oracle/ref_build.py, compiles against it).
// The models befriend boost::serialization::access and define serialize() templates; nothing in
// the reference-pin build serializes, so only the names are provided.
#pragma once

namespace boost {
namespace serialization {
class access;
template <class Base, class Derived>
Base& base_object(Derived& d) {
    return d;
}
}  // namespace serialization
}  // namespace boost

#define BOOST_CLASS_EXPORT_KEY(T)
#define BOOST_CLASS_EXPORT_IMPLEMENT(T)
#define BOOST_CLASS_EXPORT_GUID(T, K)
#define BOOST_SERIALIZATION_ASSUME_ABSTRACT(T)
