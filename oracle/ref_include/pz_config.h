/* Configuration header for compiling the NeoPZ reference sources directly
 * with g++ (oracle/ref_build.mk), in place of the header the reference's own
 * build would generate from Common/pz_config.h.in.  It sets the reference's
 * default configuration: real and state types double, no optional library
 * (LAPACK, MKL, TBB, Boost, Metis, log4cxx all off). */
#ifndef PZ_CONFIG_H_GPZ_REF
#define PZ_CONFIG_H_GPZ_REF
#ifndef PZSOURCEDIR
#define PZSOURCEDIR "."
#endif
#ifndef PZ_REFPATTERN_DIR
#define PZ_REFPATTERN_DIR "."
#endif
#ifndef PZ_BRANCH
#define PZ_BRANCH "unknown"
#endif
#ifndef PZ_REVISION
#define PZ_REVISION "unknown"
#endif
#ifndef PZ_REVISION_DATE
#define PZ_REVISION_DATE "unknown"
#endif
#ifndef PZ_LOG4CXX_CONFIG_FILE
#define PZ_LOG4CXX_CONFIG_FILE ""
#endif
#ifndef REALdouble
#define REALdouble
#endif
#ifndef STATEdouble
#define STATEdouble
#endif
#endif
