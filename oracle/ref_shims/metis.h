/* Declarations-only stand-in for METIS 5.1.0 so that Partition.C compiles.
 * Test infrastructure: Partition::PartitionGraph (the METIS path) is never
 * called by the reference's main loop (main1.C uses PartitionGraph2). */
#ifndef CAFE_REF_SHIM_METIS_H
#define CAFE_REF_SHIM_METIS_H
typedef int idx_t;
typedef float real_t;
#define METIS_NOPTIONS 40
#define METIS_OPTION_NUMBERING 17
int METIS_PartGraphRecursive(idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *,
                             idx_t *, real_t *, real_t *, idx_t *, idx_t *, idx_t *);
int METIS_PartGraphKway(idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *,
                        real_t *, real_t *, idx_t *, idx_t *, idx_t *);
#endif
