// ORACLE -- test infrastructure: FP64 radiosity placeholder (filled in with the gather oracle).
extern "C" int orc_rad_version() { return 1; }
