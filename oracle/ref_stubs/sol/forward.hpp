// Minimal forward declarations standing in for sol2, used only to compile a few of the
// reference's own translation units into oracle/_ref (no Lua is ever called).
#pragma once
namespace sol
{
class table;
class state;
} // namespace sol
