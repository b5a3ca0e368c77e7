// Test-infrastructure stub: the oracle harness compiles the reference's physics
// objects without HDF5.  output.h declares Output members of these types by value,
// so they must be complete; nothing in the harness constructs an Output.
#ifndef EPIC_ORACLE_H5CPP_STUB_H
#define EPIC_ORACLE_H5CPP_STUB_H
namespace H5 {
struct Group {};
struct H5File {};
}  // namespace H5
#endif
