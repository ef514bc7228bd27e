// Stand-in: the scenarios compiled against the facade use no generators.
#pragma once
