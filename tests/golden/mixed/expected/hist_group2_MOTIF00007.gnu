set output "hist_group2_MOTIF00007.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-46.14:15.3253]
set yrange [0:132485]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00007.dat" using 1:2 title 'MOTIF00007 (group2)' with boxes
