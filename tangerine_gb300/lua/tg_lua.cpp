// Tangerine's Lua modelling surface (tangerine/lua_sdf.cpp:223-450, the method table at
// :704-760) over this library's C ABI: a `tangerine.sdf` userdata per tree, the
// constructors and set operators as globals, and every node function also as a method.
//
// The reference's semantics are kept: sizes are diameters and are halved (sphere, box,
// cylinder, ...), n-ary union / inter / diff fold left, the blend operators take their
// threshold as the last argument, every transform or paint returns a new tree (the node is
// copied first, SDFNode::Copy), and eval / gradient / ray_cast / magnet query the whole
// tree.  Arithmetic on the arguments follows the reference's types: `luaL_checknumber(...)
// * .5` halves in double before the float conversion, vectors are read as three floats and
// halved in float.
//
// Not provided (the Tangerine application's own environment, outside the export path):
// model instancing, cameras, the background colour, materials other than a paint colour,
// stencils with a material object, random numbers and pivot_towards.  Colours are three
// numbers or "#rrggbb" strings (sRGB).
//
// The runner (main) executes a model script, takes its global `model` and prints the tree
// spec (tg_tree_spec) that rebuilds it -- the form the CPU oracle and BuildTreeFromSpec read.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

extern "C"
{
#include "lua.h"
#include "lauxlib.h"
#include "lualib.h"
}

#include "../../include/tangerine_gb300.h"

namespace
{
	const char* kSdf = "tangerine.sdf";

	void* CheckSdf(lua_State* L, int arg) { return *(void**)luaL_checkudata(L, arg, kSdf); }

	// Takes over one reference to `tree`.
	int Wrap(lua_State* L, void* tree)
	{
		if (!tree) return luaL_error(L, "tangerine: %s", tg_last_error());
		void** slot = (void**)lua_newuserdatauv(L, sizeof(void*), 0);
		*slot = tree;
		luaL_getmetatable(L, kSdf);
		lua_setmetatable(L, -2);
		return 1;
	}

	int Gc(lua_State* L)
	{
		void** slot = (void**)luaL_checkudata(L, 1, kSdf);
		if (*slot) DiscardTree(*slot);
		*slot = nullptr;
		return 0;
	}

	// GetVec3 (lua_vec.cpp:33-49): three numbers (or a table of three), each to float.
	void GetVec3(lua_State* L, int& arg, float out[3])
	{
		if (lua_istable(L, arg))
		{
			for (int i = 0; i < 3; ++i)
			{
				lua_geti(L, arg, i + 1);
				out[i] = (float)luaL_checknumber(L, -1);
				lua_pop(L, 1);
			}
			++arg;
			return;
		}
		for (int i = 0; i < 3; ++i) out[i] = (float)luaL_checknumber(L, arg++);
	}

	// A colour: three numbers or "#rrggbb" (sRGB channels in [0, 1]).
	void GetColor(lua_State* L, int& arg, float rgb[3])
	{
		if (lua_type(L, arg) == LUA_TSTRING)
		{
			const char* s = lua_tostring(L, arg++);
			unsigned v = 0;
			if (!s || s[0] != '#' || std::strlen(s) != 7 || std::sscanf(s + 1, "%6x", &v) != 1)
				luaL_error(L, "tangerine: colours are three numbers or \"#rrggbb\"");
			rgb[0] = (float)((v >> 16) & 255u) / 255.0f;
			rgb[1] = (float)((v >> 8) & 255u) / 255.0f;
			rgb[2] = (float)(v & 255u) / 255.0f;
			return;
		}
		GetVec3(L, arg, rgb);
	}

	// ---- constructors (lua_sdf.cpp:223-300) ----------------------------------------------
	int Sphere(lua_State* L) { const float r = luaL_checknumber(L, 1) * .5; return Wrap(L, MakeSphereBrush(r)); }
	int Ellipsoid(lua_State* L)
	{
		int arg = 1;
		float v[3];
		GetVec3(L, arg, v);
		return Wrap(L, MakeEllipsoidBrush(v[0] * 0.5f, v[1] * 0.5f, v[2] * 0.5f));
	}
	int Box(lua_State* L)
	{
		int arg = 1;
		float v[3];
		GetVec3(L, arg, v);
		return Wrap(L, MakeBoxBrush(v[0] * 0.5f, v[1] * 0.5f, v[2] * 0.5f));
	}
	int Cube(lua_State* L) { const float e = luaL_checknumber(L, 1) * .5; return Wrap(L, MakeBoxBrush(e, e, e)); }
	int Torus(lua_State* L)
	{
		const float major = luaL_checknumber(L, 1) * .5;
		const float minor = luaL_checknumber(L, 2) * .5;
		return Wrap(L, MakeTorusBrush(major - minor, minor));
	}
	int Cylinder(lua_State* L)
	{
		const float r = luaL_checknumber(L, 1) * .5;
		const float e = luaL_checknumber(L, 2) * .5;
		return Wrap(L, MakeCylinderBrush(r, e));
	}
	int Plane(lua_State* L)
	{
		int arg = 1;
		float n[3];
		GetVec3(L, arg, n);
		return Wrap(L, MakePlaneOperand(n[0], n[1], n[2]));
	}
	int Cone(lua_State* L)
	{
		const float r = luaL_checknumber(L, 1) * .5;
		const float h = luaL_checknumber(L, 2);
		return Wrap(L, MakeConeBrush(r, h));
	}
	int Coninder(lua_State* L)
	{
		int arg = 1;
		float v[3];
		GetVec3(L, arg, v);
		return Wrap(L, MakeConinderBrush(v[0] * 0.5f, v[1] * 0.5f, v[2] * 1.0f));
	}

	// ---- transforms and paint: on a copy (lua_sdf.cpp:56-217) -----------------------------
	void* Copied(lua_State* L) { return CopyTree(CheckSdf(L, 1)); }

	int Move(lua_State* L)
	{
		int arg = 2;
		float v[3];
		GetVec3(L, arg, v);
		void* t = Copied(L);
		MoveTree(t, v[0], v[1], v[2]);
		return Wrap(L, t);
	}
	template<int Axis>
	int MoveAxis(lua_State* L)
	{
		const float d = (float)luaL_checknumber(L, 2);
		void* t = Copied(L);
		MoveTree(t, Axis == 0 ? d : 0.0f, Axis == 1 ? d : 0.0f, Axis == 2 ? d : 0.0f);
		return Wrap(L, t);
	}
	int Align(lua_State* L)
	{
		int arg = 2;
		float v[3];
		GetVec3(L, arg, v);
		void* t = Copied(L);
		AlignTree(t, v[0], v[1], v[2]);
		return Wrap(L, t);
	}
	int Rotate(lua_State* L)
	{
		const float x = (float)luaL_checknumber(L, 2), y = (float)luaL_checknumber(L, 3);
		const float z = (float)luaL_checknumber(L, 4), w = (float)luaL_checknumber(L, 5);
		void* t = Copied(L);
		RotateTree(t, x, y, z, w);
		return Wrap(L, t);
	}
	template<int Axis>
	int RotateAxis(lua_State* L)
	{
		const float deg = (float)luaL_checknumber(L, 2);
		void* t = Copied(L);
		if (Axis == 0) RotateTreeX(t, deg);
		else if (Axis == 1) RotateTreeY(t, deg);
		else RotateTreeZ(t, deg);
		return Wrap(L, t);
	}
	int Scale(lua_State* L)
	{
		const float s = (float)luaL_checknumber(L, 2);
		void* t = Copied(L);
		ScaleTree(t, s);
		return Wrap(L, t);
	}
	int Flate(lua_State* L)
	{
		const float r = (float)luaL_checknumber(L, 2) * .5;
		return Wrap(L, MakeFlateOp(CopyTree(CheckSdf(L, 1)), r));
	}
	template<bool Force>
	int Paint(lua_State* L)
	{
		int arg = 2;
		float rgb[3];
		GetColor(L, arg, rgb);
		void* t = Copied(L);
		if (Force) PaintOverTree(rgb[0], rgb[1], rgb[2], t);
		else PaintTree(rgb[0], rgb[1], rgb[2], t);
		return Wrap(L, t);
	}

	// ---- set operators (lua_sdf.cpp:303-384): fold left over every argument ----------------
	enum class Family { Union, Inter, Diff };

	void* Combine(Family f, bool blend, float k, void* l, void* r)
	{
		switch (f)
		{
		case Family::Union: return blend ? MakeBlendUnionOp(k, l, r) : MakeUnionOp(l, r);
		case Family::Inter: return blend ? MakeBlendInterOp(k, l, r) : MakeInterOp(l, r);
		default: return blend ? MakeBlendDiffOp(k, l, r) : MakeDiffOp(l, r);
		}
	}

	template<Family F, bool Blend>
	int Operator(lua_State* L)
	{
		float k = 0.0f;
		if (Blend)
		{
			k = (float)luaL_checknumber(L, -1);
			lua_pop(L, 1);
		}
		// The operators take over their operands' references: hand them copies, as the
		// Lua values keep theirs (the reference shares the nodes; a tree is immutable once
		// a Lua value holds it, so sharing and copying give the same tree).
		void* acc = Combine(F, Blend, k, CopyTree(CheckSdf(L, 1)), CopyTree(CheckSdf(L, 2)));
		const int n = lua_gettop(L);
		for (int i = 3; i <= n; ++i) acc = Combine(F, Blend, k, acc, CopyTree(CheckSdf(L, i)));
		return Wrap(L, acc);
	}

	// ---- queries on the whole tree (lua_sdf.cpp:386-450) -----------------------------------
	int Eval(lua_State* L)
	{
		int arg = 2;
		float p[3];
		GetVec3(L, arg, p);
		lua_pushnumber(L, EvalTree(CheckSdf(L, 1), p[0], p[1], p[2]));
		return 1;
	}

	void PushVec(lua_State* L, const float v[3])
	{
		lua_createtable(L, 3, 0);
		for (int i = 0; i < 3; ++i)
		{
			lua_pushnumber(L, v[i]);
			lua_rawseti(L, -2, i + 1);
		}
	}

	int Gradient(lua_State* L)
	{
		int arg = 2;
		float p[3];
		GetVec3(L, arg, p);
		float g[3];
		GradientTree(CheckSdf(L, 1), p[0], p[1], p[2], g);
		PushVec(L, g);
		return 1;
	}

	template<bool Magnet>
	int RayCast(lua_State* L)
	{
		int arg = 2;
		float o[3], d[3];
		GetVec3(L, arg, o);
		GetVec3(L, arg, d);
		if (Magnet)
		{
			// normalize(Direction - Origin), glm order: v * inversesqrt(dot(v, v))
			const float v[3] = { d[0] - o[0], d[1] - o[1], d[2] - o[2] };
			const float s = 1.0f / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
			for (int i = 0; i < 3; ++i) d[i] = v[i] * s;
		}
		int iterations = 100;
		float epsilon = 0.001f;
		const int n = lua_gettop(L);
		if (n >= 8) iterations = (int)luaL_checkinteger(L, 8);
		if (n >= 9) epsilon = (float)luaL_checknumber(L, 9);
		const RayHit hit = RayMarchTree(CheckSdf(L, 1), o[0], o[1], o[2], d[0], d[1], d[2], iterations, epsilon);
		if (!hit.Hit)
		{
			lua_pushnil(L);
			return 1;
		}
		PushVec(L, hit.Position);
		return 1;
	}

	int Ignore(lua_State*) { return 0; }

	const luaL_Reg kFunctions[] = {
		{ "move", Move }, { "move_x", MoveAxis<0> }, { "move_y", MoveAxis<1> }, { "move_z", MoveAxis<2> },
		{ "align", Align },
		{ "rotate", Rotate }, { "rotate_x", RotateAxis<0> }, { "rotate_y", RotateAxis<1> }, { "rotate_z", RotateAxis<2> },
		{ "scale", Scale }, { "flate", Flate },
		{ "paint", Paint<false> }, { "paint_over", Paint<true> },
		{ "sphere", Sphere }, { "ellipsoid", Ellipsoid }, { "box", Box }, { "cube", Cube }, { "torus", Torus },
		{ "cylinder", Cylinder }, { "plane", Plane }, { "cone", Cone }, { "coninder", Coninder }, { "cylicone", Coninder },
		{ "union", Operator<Family::Union, false> }, { "inter", Operator<Family::Inter, false> },
		{ "diff", Operator<Family::Diff, false> },
		{ "blend_union", Operator<Family::Union, true> }, { "blend_inter", Operator<Family::Inter, true> },
		{ "blend_diff", Operator<Family::Diff, true> },
		{ "eval", Eval }, { "gradient", Gradient }, { "ray_cast", RayCast<false> }, { "magnet", RayCast<true> },
		{ "set_bg", Ignore },
		{ nullptr, nullptr },
	};

	// IndexSDFNode (lua_sdf.cpp:763-781): any function of the table is a method.
	int Index(lua_State* L)
	{
		luaL_checkudata(L, 1, kSdf);
		const char* key = luaL_checkstring(L, 2);
		for (const luaL_Reg* r = kFunctions; r->name; ++r)
		{
			if (std::strcmp(r->name, key) == 0)
			{
				lua_pushcfunction(L, r->func);
				return 1;
			}
		}
		lua_pushnil(L);
		return 1;
	}
}

extern "C" int tg_lua_open(lua_State* L)
{
	luaL_newmetatable(L, kSdf);
	lua_pushcfunction(L, Index);
	lua_setfield(L, -2, "__index");
	lua_pushcfunction(L, Gc);
	lua_setfield(L, -2, "__gc");
	lua_pop(L, 1);
	for (const luaL_Reg* r = kFunctions; r->name; ++r)
	{
		lua_pushcfunction(L, r->func);
		lua_setglobal(L, r->name);
	}
	return 0;
}

// tg_lua SCRIPT [SCRIPT...]: runs each model script in a fresh state and prints, per
// script, one line: the script path, then the words of the spec of its global `model`
// (or an error message after "error:").
int main(int argc, char** argv)
{
	int failures = 0;
	for (int a = 1; a < argc; ++a)
	{
		lua_State* L = luaL_newstate();
		luaL_openlibs(L);
		tg_lua_open(L);
		std::printf("%s", argv[a]);
		if (luaL_dofile(L, argv[a]) != LUA_OK)
		{
			std::printf(" error: %s\n", lua_tostring(L, -1));
			++failures;
		}
		else
		{
			lua_getglobal(L, "model");
			void** slot = (void**)luaL_testudata(L, -1, kSdf);
			if (!slot || !*slot)
			{
				std::printf(" error: the script sets no model\n");
				++failures;
			}
			else
			{
				const int64_t n = tg_tree_spec(*slot, nullptr, 0);
				std::vector<float> spec((size_t)(n > 0 ? n : 0));
				tg_tree_spec(*slot, spec.data(), n);
				for (float w : spec) std::printf(" %.9g", w);
				std::printf("\n");
			}
		}
		lua_close(L);
	}
	return failures ? 1 : 0;
}
