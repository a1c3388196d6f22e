// Stand-in: the planners this header names are not needed by the state space and checker it defines.
#pragma once
