// Prints the reference's OpenCL C kernel text exactly as its host code hands it to the OpenCL
// compiler (src/kernel.hpp:7-18 get_opencl_c_code(), without the device defines). Compiled by
// build_ref.py against the reference sources where they lie; test infrastructure only.
#include "kernel.cpp"

int main() {
	const std::string s = get_opencl_c_code();
	fwrite(s.data(), 1, s.size(), stdout);
	return 0;
}
