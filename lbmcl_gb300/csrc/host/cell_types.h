// cell_types.h -- the reference's integer cell-type flags (common.h:7-20)
// and the predicates its map dump uses (common.h:23-66, lbmcl.hpp:188-193).
// lbm_dump(LBM_DUMP_MAP) returns these values.
#pragma once

namespace lbmcl {

enum CellFlag : int {
    CELL_NONE = 0x000,
    CELL_FLUID = 0x001,
    CELL_MOVING = 0x002,
    CELL_CORNER = 0x004,
    CELL_WALL = 0x008,
    CELL_LEFT = 0x010,
    CELL_RIGHT = 0x020,
    CELL_TOP = 0x040,
    CELL_BOTTOM = 0x080,
    CELL_FRONT = 0x100,
    CELL_BACK = 0x200,
};

inline bool cell_is_fluid(int c) { return c == CELL_FLUID; }
inline bool cell_is_wall(int c) { return c == CELL_WALL; }
inline bool cell_is_corner(int c) { return c == CELL_CORNER; }
inline bool cell_is_moving(int c) { return (c & CELL_MOVING) != 0; }
inline bool cell_is_boundary(int c)
{
    return (c & (CELL_LEFT | CELL_RIGHT | CELL_BOTTOM | CELL_TOP | CELL_BACK | CELL_FRONT)) != 0;
}

// Map-dump code: FLUID 1, MOVING 2, BOUNDARY 3, WALL 4, CORNER 5, the later
// test winning (lbmcl.hpp:188-193).
inline int cell_dump_code(int c)
{
    int v = 0;
    if (cell_is_fluid(c)) v = 1;
    if (cell_is_moving(c)) v = 2;
    if (cell_is_boundary(c)) v = 3;
    if (cell_is_wall(c)) v = 4;
    if (cell_is_corner(c)) v = 5;
    return v;
}

}  // namespace lbmcl
