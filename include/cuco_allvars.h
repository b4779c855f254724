/* cuco_allvars.h - the reference's data types, as the drop-in sees them.
 *
 * The drop-in entry points of libcuco_gb300.so read and write the reference
 * host program's globals (P, NumPart, All, header, the drift tables and the
 * gravlist device pointers).  These declarations restate the reference's own
 * types field for field, because the layout is an ABI that must match:
 *   PARTICLE  allvars.h:35-45  (60 bytes)
 *   HEADER    allvars.h:47-57  (32 bytes; also the snapshot/IC file header)
 *   ALL       allvars.h:59-118
 *   SIMPARAM  proto.cuh:7-18,  SOFTPARAM proto.cuh:20-24
 * The sizes and field offsets are checked against the reference build by the
 * CPU tests (tests/test_abi.py).  A host program that keeps the reference's
 * allvars.h/allvars.c includes its own header instead of this one. */
#ifndef CUCO_ALLVARS_H
#define CUCO_ALLVARS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUCO_TIMEBASE (1 << 28)            /* allvars.h:11 */
#define CUCO_ASMTH 1.25                    /* allvars.h:24 */
#define CUCO_RCUT 4.5                      /* allvars.h:25 */
#define CUCO_NTAB 1000                     /* allvars.h:27 */
#define CUCO_DRIFT_TABLE_LENGTH 1000       /* allvars.h:29 */
#define CUCO_MAXLEN_OUTPUTLIST 500         /* allvars.h:30 */
#define CUCO_MAXLEN_FILENAME 250           /* allvars.h:31 */

typedef struct particle_data {
    float Pos[3];
    float Mass;
    float Vel[3];
    float GravAccel[3];
    float GravPM[3];
    int Ti_endstep;
    int Ti_begstep;
} PARTICLE;

typedef struct io_header {
    int NumPart;
    float Mass;
    float Time;
    float Redshift;
    float BoxSize;
    float Omega0;
    float OmegaLambda;
    float HubbleParam;
} HEADER;

typedef struct global_data {
    int NumPart;
    float BoxSize;
    float Mass;
    double G;
    double UnitTime_in_s;
    double UnitMass_in_kg;
    double UnitVelocity_in_m_per_s;
    double UnitLength_in_m;
    double UnitTime_in_Megayears;
    float Hubble;
    float Omega0;
    float OmegaLambda;
    float OmegaBaryon;
    float HubbleParam;
    float Time;
    float TimeBegin;
    float TimeStep;
    float TimeMax;
    double Timebase_interval;
    int Ti_Current;
    int Ti_nextoutput;
    int PM_Ti_endstep;
    int PM_Ti_begstep;
    float Asmth;
    float Rcut;
    float ErrTolIntAccuracy;
    float MaxSizeTimestep;
    float MinSizeTimestep;
    float SofteningHalo;
    float SofteningHaloMaxPhys;
    float SofteningTable;
    float ForceSoftening;
    int NumCurrentTiStep;
    int SnapshotFileCount;
    float OutputListTimes[CUCO_MAXLEN_OUTPUTLIST];
    int OutputListLength;
    char InitCondFile[CUCO_MAXLEN_FILENAME];
    char OutputDir[CUCO_MAXLEN_FILENAME];
    char SnapshotFileBase[CUCO_MAXLEN_FILENAME];
    char OutputListFilename[CUCO_MAXLEN_FILENAME];
} ALL;

typedef struct tagSimParam {
    float shortrange_table[CUCO_NTAB];
    float boxsize;
    float boxhalf;
    float to_grid_fac;
    float rcut;
    float rcut2;
    float asmth;
    float asmthfac;
    float mass;
    float G;
} SIMPARAM;

typedef struct tagSoftParam {
    float h;
    float h_inv;
    float h3_inv;
} SOFTPARAM;

#ifdef __cplusplus
}
#endif
#endif
