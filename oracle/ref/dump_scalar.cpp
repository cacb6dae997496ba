// Output_Scalar (lib/structure/s_io_file.hpp:43-71) ends without returning
// its int; g++ treats the end of such a function as unreachable (a trap at
// -O0, undefined code at -O2) and the call crashes. This translation unit
// instantiates it alone and is compiled with -O0 -fno-unreachable-traps,
// where the function simply returns (the caller ignores the value).
// Formatting is done by the reference's fmt, so the file is byte for byte
// what the reference writes.
#include "structure/s_io_file.hpp"

void harness_output_scalar(const std::string& filename,
		const structure::Scalar_<2>& s) {
	structure::Output_Scalar(filename, s);
}
