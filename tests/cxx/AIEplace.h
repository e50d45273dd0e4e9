// Stand-in for the reference host's AIEplace.h (vck5000/host/src/include):
// only the members the INTEGRATION.md binding touches, with the reference's
// names and types (AIEplace.h:21-99, DataBase.h:103-105, Node.h:19-126,
// Net.h:54, Grid.h:34-35, Position.h), so that the binding is compiled
// against the interface it will meet.  Test infrastructure.
#pragma once
#include <cstdlib>
#include <iostream>  // the reference header brings these in through Common.h
#include <map>
#include <string>
#include <vector>

namespace AIEplace {

enum PlacementStatus { UNPLACED = 0x0, PLACED = 0x1, FIXED = 0x2, DUMMY_FIXED = 0x3, UNKNOWN = 0x4 };

template <typename T>
class Position {
  public:
    Position(T x = 0, T y = 0) : x_(x), y_(y) {}
    const T &getX() const { return x_; }
    const T &getY() const { return y_; }

  private:
    T x_, y_;
};

class Node {
  public:
    virtual ~Node() = default;
    const PlacementStatus &getStatus() { return status_; }
    const float &getX() { return pos_.getX(); }
    const float &getY() { return pos_.getY(); }
    void setPosition(Position<float> p) { pos_ = p; }
    virtual float getXsize() { return 0.0; }
    virtual float getYsize() { return 0.0; }

  private:
    PlacementStatus status_ = UNPLACED;
    Position<float> pos_;
};

class Component : public Node {};
class Pin : public Node {};

class Net {
  public:
    const std::vector<Node *> &getNodes() { return nodes_; }

  private:
    std::vector<Node *> nodes_;
};

class DataBase {
  public:
    const std::map<std::string, Component *> &getComponents() { return components_; }
    const std::map<std::string, Pin *> &getPins() { return pins_; }
    const std::map<std::string, Net *> &getNets() { return nets_; }

  private:
    std::map<std::string, Component *> components_;
    std::map<std::string, Pin *> pins_;
    std::map<std::string, Net *> nets_;
};

class Grid {
  public:
    int getDieWidth() { return 0; }
    int getDieHeight() { return 0; }
};

class Placer {
  public:
    DataBase db;
    Grid grid;
    int bins_per_row = 512;
};

}  // namespace AIEplace
