// Stand-in: the benchmark tool is not needed by the state space and checker the demo header defines.
#pragma once
