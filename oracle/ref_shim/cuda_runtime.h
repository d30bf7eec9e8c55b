// Stand-in: StatTile needs nothing from the CUDA runtime header.
#pragma once
