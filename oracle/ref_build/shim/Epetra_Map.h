/* Stand-in declaration for Epetra_Map.h (Trilinos): the maps are named by
 * reference headers, never used on the paths the harnesses reach.  Test
 * infrastructure only. */
#ifndef XG_SHIM_EPETRA_MAP
#define XG_SHIM_EPETRA_MAP
class Epetra_BlockMap;
class Epetra_Map;
#endif
