set output "hist_cfg1_MOTIF00029.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-89.2771:20.8981]
set yrange [0:178291]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00029.dat" using 1:2 title 'MOTIF00029 (cfg1)' with boxes
