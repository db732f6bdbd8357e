/* Oracle build of the reference, 1D, shipped constants (no overrides).
 * Force-included after parameters.h by oracle/Makefile. */
