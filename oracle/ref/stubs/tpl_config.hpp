/* Third-party configuration for the single-rank oracle build of the reference. */
#define OCP_USE_MPI
