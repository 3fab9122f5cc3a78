// ref_stubs.cpp -- link-time stand-in for the reference LBS kernel's host stub.
// examples/load_balanced_search/lbs.cu's main() (renamed, never called) launches
// extract_edges_block; the kernel is not built for the CPU checker executable,
// and the linker cannot leave a hidden kernel-stub symbol unresolved.
void extract_edges_block(int, int *, int *, int *, int *) {}
