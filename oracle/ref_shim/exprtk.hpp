// Empty stand-ins for the expression-library types the reference's
// MathCode.h names as members.  Loads in the oracle are table-driven; the
// expression path (MathCode.cpp) is not linked.
#pragma once
namespace exprtk {
template <typename T> struct symbol_table {};
template <typename T> struct expression {};
template <typename T> struct parser {};
}  // namespace exprtk
