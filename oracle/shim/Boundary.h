/* Wall conditions of the checker build: free slip on all six velocity walls
   (the configurations' "free-slip walls"), in the macro form of the
   reference's Include/Boundary.h. */
#ifndef H_BOUNDARY
#define H_BOUNDARY
#define BACK_WALL_VELOCITY_FREESLIP
#define FRONT_WALL_VELOCITY_FREESLIP
#define BOTTOM_WALL_VELOCITY_FREESLIP
#define TOP_WALL_VELOCITY_FREESLIP
#define LEFT_WALL_VELOCITY_FREESLIP
#define RIGHT_WALL_VELOCITY_FREESLIP
/* as in the reference Boundary.h: not a driven-cavity case */
#undef DRIVEN_CAVITY
#endif
